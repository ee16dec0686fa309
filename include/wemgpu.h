/*
 * wemgpu.h — C ABI of the GB300 one-way wave-equation library.
 *
 * Drop-in boundary for the one-way downward-continuation hot path of
 * arustam92/wem-fwi (split-step Fourier / PSPI depth step and the Born
 * operators built on it).  Every entry point replaces one binding of the
 * reference's pybind11 modules; the replaced interface is cited beside it.
 *
 * Conventions
 *   - complex values are interleaved float pairs (re, im), C99-compatible
 *     with `float _Complex` and `std::complex<float>`;
 *   - 2D fields are row-major [nz][nx] with x fastest, the layout of the
 *     reference's complex2DReg::_mat (complex/include/complex2DReg.h:41-46);
 *   - frequency-extended fields are [nw][nz][nx];
 *   - data are [ns][nr][nt] (real, time) or [ns][nr][nbin] (complex bins),
 *     time/bin fastest, as in the reference's float3DReg / complex3DReg;
 *   - pointers may be host or device memory; the library detects which and
 *     moves host buffers itself (host calls are synchronous);
 *   - `add` follows the reference: 0 zeroes the output before accumulating;
 *   - no C++ exception crosses this boundary: every call returns a status
 *     code; wem_last_error() gives the message of the last failure on the
 *     calling thread.
 *
 * Threading: a handle is not thread-safe; use one handle per host thread /
 * CUDA stream.  The reference drives one operator object per Python process
 * and holds the GIL around every call (propagator/src/python/pyWEM.cpp).
 */
#ifndef WEMGPU_H
#define WEMGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  WEM_OK       = 0,
  WEM_EINVAL   = 1,  /* bad argument: shape, geometry, parameter, slowness <= 0 */
  WEM_ENOMEM   = 2,  /* device or host allocation failed */
  WEM_EDEVICE  = 3,  /* CUDA error reported by the runtime */
  WEM_ETIMEOUT = 4,  /* a bounded device wait ran out (error word set by a kernel) */
  WEM_ENOTIMPL = 5   /* valid request this build does not support */
};

/* propagator choice: par "prop" (propagator/src/OneWay.cpp:22-27) */
enum { WEM_PROP_SSF = 0, WEM_PROP_PSPI = 1 };

/* adjoint flavour of the Born operators.
 * COMPAT reproduces the reference's adjoint exactly as coded: Scatter's
 *   k-filter applied before the slowness scaling (propagator/src/Scatter.cpp:52-66)
 *   and LinDown::adjoint clearing the last depth row of the gradient
 *   (propagator/src/LinOneWay.cpp:64-65), with the frequencies of one shot
 *   processed in order by one task.
 * EXACT is the true transpose of the forward operator (dot test to 1e-5). */
enum { WEM_ADJ_COMPAT = 0, WEM_ADJ_EXACT = 1 };

/* reference-slowness partition (propagator/src/RefSampler.cpp:41-84).
 * ASCODED replays the reference's sort of the nx-long history buffer;
 * NEAREST is the textbook nearest-reference partition. */
enum { WEM_REFS_ASCODED = 0, WEM_REFS_NEAREST = 1 };

/* phase law of the phase shift (kernel of Phshift, a1).
 * ISPC is the propagator's law (phase_shift.ispc:2-32): re/im of the damped
 * square root of w^2 (s - i eps Re s) - k^2.  EXACT_KZ is the law of the
 * older extPropagator (extPropagator/src/Phshift.cpp:41-126): forward factor
 * exp(-i dz conj(kz)), kz = sqrt(w^2 s - k^2 + 1e-5 i), on the same k grid. */
enum { WEM_PHASE_ISPC = 0, WEM_PHASE_EXACT_KZ = 1 };

/* data representation of a call */
enum { WEM_DATA_TIME = 0,    /* float  [ns][nr][nt]                         */
       WEM_DATA_FREQ = 1 };  /* complex [ns][nr][nbin] (nbin >= nt + tpad) */

/* Parameters.  Names and defaults follow the reference's paramObj keys
 * (PropParam.h:45-85, OneStep.h:19-38, Device.h:39-85, wem_prop.cpp:43-44,
 * LinOneWay.cpp:17, Scatter.cpp:12).  wem_params_default() fills defaults. */
typedef struct wem_params {
  /* model grid: axis 1 = x (fast), axis 2 = z */
  int   nx, nz;
  float ox, oz, dx, dz;
  /* wavelet / data time axis */
  int   nt;
  float ot, dt;
  /* regular acquisition (Device.h:39-63) */
  int   ns;  float osx, osz, dsx, dsz;
  int   nr;  float orx, orz, drx, drz;
  /* irregular acquisition (Device.h:65-85): when non-NULL these coordinate
   * arrays (ns resp. nr entries) replace the regular geometry above */
  const float* src_x; const float* src_z;
  const float* rec_x; const float* rec_z;
  /* propagation */
  int   prop;      /* WEM_PROP_SSF | WEM_PROP_PSPI            ("prop")    */
  int   nref;      /* reference slownesses, default 1         ("nref")    */
  int   tap;       /* FFT zero pad each side, default 0       ("tap")     */
  int   pad;       /* model edge pad + taper width, default 0 ("pad")     */
  int   tpad;      /* time zero pad at the end, default 0     ("tpad")    */
  int   ngs, ngr;  /* cos^2 source / receiver half widths     ("ngs","ngr")*/
  int   ntaylor;   /* Taylor terms of the Born scatter, default 1, max 4 */
  float eps;       /* evanescent damping, default 0.04        ("eps")     */
  float fmin;      /* default 1                               ("fmin")    */
  float fmax;      /* default 0 (then nfreq bins from bin 1)  ("fmax")    */
  int   nfreq;     /* used when fmax == 0, default 0          ("nfreq")   */
  /* choices that have no reference key */
  int   adjoint_mode;  /* WEM_ADJ_COMPAT (default) | WEM_ADJ_EXACT */
  int   refs_mode;     /* WEM_REFS_ASCODED (default) | WEM_REFS_NEAREST */
  int   nbin;          /* bins of WEM_DATA_FREQ data; 0 = nt + tpad */
  int   phase_law;     /* WEM_PHASE_ISPC (default) | WEM_PHASE_EXACT_KZ */
  /* conformal-map geometry of WEM and BornFull, one map per shot
   * (PropParam.h:88-137; conformal/src): every shot propagates in its own
   * mapped coordinates ("cmap").
   *   WEM_CMAP_NONE  identity (Identity.h), the default;
   *   WEM_CMAP_LOG   shift-and-scale onto the unit disc around the source
   *                  followed by the complex logarithm with inner radius
   *                  eps_log (ShiftAndScale.h, ComplexLog.h/.cpp): the source
   *                  becomes a line along the first mapped depth;
   *   WEM_CMAP_ROT   rotation of the grid by cmap_angles[is] radians
   *                  (Rotation.h), ns angles (the reference reads them from
   *                  the JSON file named by "cmap_angles", key "a"). */
  int   cmap;
  float eps_log;              /* default 0.01 ("eps_log") */
  const float* cmap_angles;   /* ns angles for WEM_CMAP_ROT */
} wem_params;

enum { WEM_CMAP_NONE = 0, WEM_CMAP_LOG = 1, WEM_CMAP_ROT = 2 };

void wem_params_default(wem_params* p);

/* number of propagated frequencies for these parameters
 * (PropParam::get_nfreq, PropParam.h:42; pyWEM.cpp:36-39) */
int wem_count_freqs(const wem_params* p, const float* wavelet, int* nfreq);

const char* wem_last_error(void);
const char* wem_version(void);

/* Kernel timing (no counterpart in the reference: measurement support).
 * While enabled, every pass kernel is bracketed by CUDA events on the stream
 * it is launched on; per-kernel totals accumulate until reset.  Kernel names:
 * "k_wem", "k_born_fwd", "k_born_adj", "k_wem_grad"; the offset Born's
 * "k_off_down", "k_off_up", "k_off_upadj" (one sweep over every row, all its
 * launches), "k_off_source", "k_off_image". */
int wem_stats_enable(int on);
int wem_stats_get(const char* kernel, double* total_ms, long long* launches);
int wem_stats_reset(void);
/* Number of kernel launches the library has made in this process (all
 * kernels, every entry point); never reset. */
long long wem_launch_count(void);

/* Launch shape (no counterpart in the reference: measurement support).
 * plain = 1 runs every (shot, frequency) row as its own kernel launch, one
 * CTA per launch: the unbatched GPU form the batched path is compared with.
 * plain = 0 (default) runs all groups of rows in one launch per pass. */
int wem_set_plain(int plain);

/* Kernel family (no counterpart in the reference: test and measurement
 * support).  0 automatic (warp-per-row kernels when N = 32 E with E in
 * {8, 12, 16, 24, 32}, shared-memory kernels otherwise), 1 shared-memory
 * kernels only, 2 warp-per-row kernels only (WEM_EINVAL when N is not
 * supported). */
int wem_set_kernel_path(int path);

/* Rows per CTA of the single-reference warp-per-row kernels (no counterpart
 * in the reference: launch shape).  0 automatic (one row per CTA when a pass
 * has no more (shot, frequency) rows than the GPU has SMs, rows of a
 * frequency grouped per CTA otherwise), 1 grouped rows, 2 one row per CTA.
 * Results do not depend on it beyond float rounding of the image sums. */
int wem_set_row_ctas(int mode);

/* Source field of fwi_gradient (no counterpart in the reference: pass
 * structure).  1 (default): where both passes run in one launch of the
 * grouped warp kernels, the modelling pass stores the down-going source
 * field and the Born adjoint reuses it instead of recomputing it; 0: the
 * Born adjoint recomputes it.  Results differ by float rounding only;
 * WEM_EINVAL for other values. */
int wem_set_gradient_split(int on);

/* ------------------------------------------------ nonlinear modelling (WEM) */
typedef struct wem_handle wem_handle;

/* replaces pyWEM.WEM(float1DReg wave, hypercube, paramObj)
 * (propagator/src/python/pyWEM.cpp:21-23; WEMnl.cpp:11-21) */
int wem_create(const wem_params* p, const float* wavelet, wem_handle** out);
void wem_destroy(wem_handle* h);
int wem_get_nfreq(wem_handle* h, int* nfreq);

/* replaces WEM::forward(vector<complex2DReg> [s2, rho], float3DReg | complex3DReg, add)
 * (WEMnl.cpp:39-82; wem_prop.cpp:9-78).  slow2/rho: complex [nz][nx];
 * data: kind WEM_DATA_TIME (float) or WEM_DATA_FREQ (complex). */
int wem_forward(wem_handle* h, const void* slow2, const void* rho,
                void* data, int data_kind, int add);

/* -------------------------------------------------- Born operator (BornFull) */
typedef struct born_handle born_handle;

/* replaces pyWEM.Born(float1DReg wave, vector<complex2DReg> [s2, rho], paramObj)
 * (pyWEM.cpp:45-47; BornFull.cpp:13-37) */
int born_create(const wem_params* p, const float* wavelet,
                const void* bg_slow2, const void* bg_rho, born_handle** out);
void born_destroy(born_handle* h);
/* replaces BornFull::setBgSlow (BornFull.h:24-29; pyWEM.cpp:67-69) */
int born_set_background(born_handle* h, const void* bg_slow2, const void* bg_rho);
/* replaces BornFull::forward (BornFull.cpp:39-78; born_prop.cpp:11-116) */
int born_forward(born_handle* h, const void* dslow2, const void* drho,
                 void* data, int data_kind, int add);
/* replaces BornFull::adjoint (BornFull.cpp:80-117; born_prop.cpp:119-235) */
int born_adjoint(born_handle* h, void* dslow2, void* drho,
                 const void* data, int data_kind, int add);

/* ---------------------------------- frequency-extended Born variants
 * BornRefl: replaces pyWEM.BornRefl (pyWEM.cpp:83-97; BornRefl.cpp,
 * ext_born_refl.cpp:8-105).  model: complex [nfreq][nz][nx] reflectivity
 * per frequency; forward records Up(bg m_f), adjoint gives the image
 * sum over shots of conj(bg) Up^H(data) per frequency.
 * BornTomo: replaces pyWEM.BornTomo (pyWEM.cpp:101-115; BornTomo.cpp,
 * ext_born_tomo.cpp:9-119).  model: complex [nz][nx] slowness^2
 * perturbation; the down- and up-scattering terms of BornFull with the
 * reflectivity set by borntomo_set_refl ([nfreq][nz][nx]) in place of R.
 * Backgrounds are slowness^2 only (the reference takes no density).
 * Both keep the reference's conventions for these classes, which differ
 * from BornFull's (ext_born_refl.cpp:18-25, ext_born_tomo.cpp:20-25): they
 * propagate on the model grid itself (no edge padding; p->pad is only the
 * taper width of OneStep.h:27-35), the source spreads over p->ngs cells
 * (the reference's parameter "ng") and the receivers are points (p->ngr is
 * not read). */
typedef struct bornrefl_handle bornrefl_handle;
int bornrefl_create(const wem_params* p, const float* wavelet, const void* bg_slow2, bornrefl_handle** out);
void bornrefl_destroy(bornrefl_handle* h);
/* replaces BornRefl::setBgSlow (BornRefl.h:25-29) */
int bornrefl_set_background(bornrefl_handle* h, const void* bg_slow2);
int bornrefl_forward(bornrefl_handle* h, const void* model, void* data, int data_kind, int add);
int bornrefl_adjoint(bornrefl_handle* h, void* model, const void* data, int data_kind, int add);

/* Subsurface-offset extended reflectivity Born (no reference counterpart;
 * the extension the reference's BornRefl, propagator/src/ext_born_refl.cpp:
 * 8-105, and IC, propagator/src/ic.cpp:5-29, reduce from at one lag).
 * Model r [nh][nz][nx] complex64: the reflectivity at horizontal lag
 * l = i - (nh - 1)/2 grid cells (nh odd, <= 41).  Per (shot, frequency):
 *   forward  bg = Down(src); sc(x) = sum_l r_l(x - l) bg(x - 2l); record Up(sc)
 *   adjoint  bg = Down(src); a = Up^H(data); image_l(x) += conj(bg(x - l)) a(x + l)
 * Shot s propagates on its aperture, model columns [ap_x0[s], ap_x0[s] +
 * ap_w[s]) (even widths; NULL: the whole model for every shot), with
 * BornRefl's conventions (no edge padding, pad the taper width, source
 * spread ngs, point receivers), zero-padded to the row length N_s, the
 * smallest of 256, 384, 512, 768, 1024 with N_s >= ap_w[s] + 2 tap, equally
 * on both sides (bornoff_rows reports N_s and the leading zero pad).  The aperture is a
 * cropped model as WEM.from_subspace builds it (propagator/src/python/
 * WEM.py:24-30): the reference slowness comes from the aperture, receivers
 * outside it record zero and are ignored by the adjoint.  One reference
 * slowness (nref = 1), SSF or PSPI; background slowness^2 with unit
 * density.  With nh = 1 and full apertures the operator is BornRefl with
 * the same reflectivity at every frequency, summed over frequencies in the
 * adjoint. */
typedef struct bornoff_handle bornoff_handle;
int bornoff_create(const wem_params* p, const float* wavelet, const void* bg_slow2, int nh, const int* ap_x0,
                   const int* ap_w, bornoff_handle** out);
void bornoff_destroy(bornoff_handle* h);
int bornoff_set_background(bornoff_handle* h, const void* bg_slow2);
int bornoff_forward(bornoff_handle* h, const void* model, void* data, int data_kind, int add);
int bornoff_adjoint(bornoff_handle* h, void* model, const void* data, int data_kind, int add);
int bornoff_rows(bornoff_handle* h, int* row_len, int* tap);

/* 3D one-way operators on planes (no reference counterpart: the reference
 * propagates 2D slices; at ny = 1 these are WEM, propagator/src/
 * wem_prop.cpp:9-78, and BornRefl, ext_born_refl.cpp:8-105).  The depth step
 * is the reference's SSF / PSPI step (SSF.cpp:8-60, PSPI.cpp:8-53) with a 2D
 * FFT of each depth slice and k^2 = kx^2 + ky^2 in the phase shift
 * (phase_shift.ispc:2-16); the taper is the product of the x and y tapers;
 * RefSampler (RefSampler.cpp:10-91) runs on each slice flattened row by row
 * (y-major); sources and receivers spread along x only (ngs, ngr).
 * Models are [nz][ny][nx] complex64; data [ns][nr][nt] (time) or
 * [ns][nr][nbin] (bins) as in 2D.  Row lengths: nx + 2 pad + 2 tap and
 * ny + 2 pad_y + 2 tap_y each in {256, 384, 512, 768, 1024}, or ny = 1 with
 * no y padding.  The reflectivity Born pair (refl3d_*) keeps BornRefl's
 * conventions: no edge padding (pad and pad_y are taper widths only, so
 * nx + 2 tap and ny + 2 tap_y are the row lengths) and point receivers.
 * checkpoint k > 1 keeps the down field every k depths and recomputes the
 * segments between in the up sweep (the same numbers). */
typedef struct wem3d_params {
  wem_params p;          /* x, z and time axes, propagation; device coordinates
                            p.src_x/src_z (ns) and p.rec_x/rec_z (nr) required */
  int ny;
  float oy, dy;
  int pad_y, tap_y;      /* edge pad + taper width, FFT zero pad along y */
  const float* src_y;    /* ns */
  const float* rec_y;    /* nr */
} wem3d_params;
typedef struct wem3d_handle wem3d_handle;
int wem3d_create(const wem3d_params* p, const float* wavelet, wem3d_handle** out);
void wem3d_destroy(wem3d_handle* h);
int wem3d_get_nfreq(wem3d_handle* h, int* nfreq);
int wem3d_forward(wem3d_handle* h, const void* slow2, const void* rho, void* data, int data_kind, int add,
                  int checkpoint);
typedef struct refl3d_handle refl3d_handle;
int refl3d_create(const wem3d_params* p, const float* wavelet, const void* bg_slow2, refl3d_handle** out);
void refl3d_destroy(refl3d_handle* h);
int refl3d_set_background(refl3d_handle* h, const void* bg_slow2);
int refl3d_forward(refl3d_handle* h, const void* model, void* data, int data_kind, int add, int checkpoint);
int refl3d_adjoint(refl3d_handle* h, void* model, const void* data, int data_kind, int add);

typedef struct borntomo_handle borntomo_handle;
int borntomo_create(const wem_params* p, const float* wavelet, const void* bg_slow2, borntomo_handle** out);
void borntomo_destroy(borntomo_handle* h);
/* replaces BornTomo::setBgSlow / setBgRefl (BornTomo.h:36-43) */
int borntomo_set_background(borntomo_handle* h, const void* bg_slow2);
int borntomo_set_refl(borntomo_handle* h, const void* refl);
int borntomo_forward(borntomo_handle* h, const void* dslow2, void* data, int data_kind, int add);
int borntomo_adjoint(borntomo_handle* h, void* dslow2, const void* data, int data_kind, int add);

/* ------------------------------------------ FWI objective and gradient
 * No single reference counterpart: one call for what scripts/fwi.py:70-71,90
 * composes from NonLinearOperator(wemOp, bornOp) and the solver's L2
 * residual (python-solver ProblemL2NonLinear):
 *   loss = 1/2 ||WEM(s2, rho) - d_obs||^2
 *   (g_slow2, g_rho) = Born^H(WEM(s2, rho) - d_obs) at the background (s2, rho)
 * with the parameters' adjoint_mode (compat: the reference's gradient as
 * coded).  d_obs: float [ns][nr][nt] time traces.  Host or device pointers.
 * The residual and the loss stay on the device, and the tables of the
 * background are built once for both passes. */
typedef struct fwi_handle fwi_handle;
int fwi_create(const wem_params* p, const float* wavelet, fwi_handle** out);
void fwi_destroy(fwi_handle* h);
int fwi_gradient(fwi_handle* h, const void* slow2, const void* rho, const void* d_obs,
                 void* g_slow2, void* g_rho, double* loss);

/* ---------------------------------- exact gradient of the nonlinear modelling
 * No reference counterpart: the reference's FWI gradient is the Born adjoint
 * above (a Taylor-scatter linearisation that holds the reference slownesses
 * fixed and scales dReflect as dReflect.h:18-24 codes it), which is not the
 * derivative of its modelled data.  These differentiate WEM::forward
 * (wem_prop.cpp:9-78, WEMnl.cpp:11-82) exactly: through Reflect
 * (Reflect.h:12-48), the split step (SplitStep.cpp:5-29), the phase shift
 * (phase_shift.ispc:2-32, or the exact-kz law) and the reference slowness
 * that RefSampler samples from the model (RefSampler.cpp:28-39).  The
 * gradient of a real function L of the data is returned as
 * dL/dRe + i dL/dIm for each complex model value.
 * Requires one reference (nref = 1, SSF or PSPI), no conformal map, and
 * N = nx + 2 pad + 2 tap = 32 E with E in {8, 12, 16, 24, 32}
 * (WEM_ENOTIMPL otherwise).  checkpoint: 0 or 1 keeps every depth's
 * wavefields on the device; k > 1 keeps every k-th depth and recomputes the
 * k depths between from it (the same numbers, bit for bit; about 4/10 more
 * work), which divides the stored bytes by about k.
 *
 * fwi_gradient_exact: loss = 1/2 ||WEM(s2, rho) - d_obs||^2 (d_obs float
 * [ns][nr][nt]) and its exact gradient.
 * wem_gradient: (g_slow2, g_rho) (+)= J^H g for the derivative J of
 * wem_forward at (slow2, rho) and a data gradient g (data_kind as
 * wem_forward: float time traces or complex bins). */
int fwi_gradient_exact(fwi_handle* h, const void* slow2, const void* rho, const void* d_obs,
                       void* g_slow2, void* g_rho, double* loss, int checkpoint);
int wem_gradient(wem_handle* h, const void* slow2, const void* rho, const void* data_grad,
                 int data_kind, void* g_slow2, void* g_rho, int add, int checkpoint);

/* ------------------------------------- frequency-extended operators (ext*) */
typedef struct extwem_handle extwem_handle;
typedef struct extborn_handle extborn_handle;

/* replaces pyWEM.extWEM (pyWEM.cpp:142-156; extWEM.cpp:9-70; ext_wem_prop.cpp:8-59).
 * model: complex [nfreq][nz][nx] slowness^2 and density. */
int extwem_create(const wem_params* p, const float* wavelet, extwem_handle** out);
void extwem_destroy(extwem_handle* h);
int extwem_forward(extwem_handle* h, const void* slow2, const void* rho,
                   void* data, int data_kind, int add);

/* replaces pyWEM.extBorn (pyWEM.cpp:159-186; extBornFull.cpp:11-121;
 * ext_born_prop.cpp:8-194) */
int extborn_create(const wem_params* p, const float* wavelet,
                   const void* bg_slow2, const void* bg_rho, extborn_handle** out);
void extborn_destroy(extborn_handle* h);
int extborn_set_background(extborn_handle* h, const void* bg_slow2, const void* bg_rho);
int extborn_forward(extborn_handle* h, const void* dslow2, const void* drho,
                    void* data, int data_kind, int add);
int extborn_adjoint(extborn_handle* h, void* dslow2, void* drho,
                    const void* data, int data_kind, int add);

/* --------------------------------------------- row-level operators (wem_ops)
 * Batched forms of the per-row operators that py_wem_ops binds
 * (propagator/src/python/py_wem_ops.cpp:24-208, wem_ops.py:6-137).
 * A wemop handle holds one padded background slowness [nz][nxg] (nxg =
 * nx + 2 pad, already edge padded, as the drivers pass it) and the
 * RefSampler built on it. */
typedef struct wemop_handle wemop_handle;

int wemop_create(const wem_params* p, const void* slow_padded, int nxg,
                 wemop_handle** out);
void wemop_destroy(wemop_handle* h);

/* SSF / PSPI depth step of nrow rows [nrow][nxg] at depth iz, frequency
 * freq (Hz).  Replaces SSF::forward/adjoint and PSPI::forward/adjoint
 * (SSF.cpp:8-60, PSPI.cpp:8-53).  adj=0: out = P in; adj=1: out = P^H in. */
int wemop_onestep(wemop_handle* h, int iz, float freq, int adj,
                  const void* in, void* out, int nrow, int add);

/* Down / Up over whole fields [nrow][nz][nxg].  Replaces Down/Up::forward /
 * adjoint (OneWay.cpp:32-109).  up=0: Down, up=1: Up.  When in == out the
 * call is the in-place recursion the drivers use; otherwise the reference's
 * out-of-place single-step semantics apply. */
int wemop_oneway(wemop_handle* h, int up, float freq, int adj,
                 const void* in, void* out, int nrow, int add);

/* Taylor Born scatter of nrow rows at depth iz.  Replaces
 * Scatter::forward/adjoint (Scatter.cpp:35-66); the adjoint flavour follows
 * the handle's adjoint_mode. */
int wemop_scatter(wemop_handle* h, int iz, float freq, int adj,
                  const void* in, void* out, int nrow, int add);

/* Reference slownesses [nz][nref] (complex) and the reference index of each
 * grid point [nz][nxg] (-1 = no reference) of the handle's RefSampler.
 * Replaces RefSampler::getRefSlow / getRefLoc (RefSampler.h:19-20). */
int wemop_refsampler(wemop_handle* h, void* sref, int* refidx);

/* SplitStep of one depth on the listed points (propagator/src/SplitStep.cpp:5-29;
 * py_wem_ops.cpp SplitStep, setFreq/setLocation/setSlow/setDepth): point x
 * of each row gets m[x] exp(-i w dz (s[iz][x] - sref) / sqrt(sref)) (adjoint
 * exp(+i w dz conj(...))), s the handle's slowness^2, dz its p.dz.  As in the
 * reference the listed points are assigned, not accumulated; the other
 * points are zero without add and untouched with it.  in, out [nrow][nxg]. */
int wemop_splitstep(wemop_handle* h, int iz, float freq, float sref_re, float sref_im,
                    const int* loc, int nloc, int adj, const void* in, void* out,
                    int nrow, int add);
/* LinDown of one field [nz][nxg] with the background wavefield bg [nz][nxg]
 * (LinOneWay.cpp:33-85; py_wem_ops.cpp LinDown): per depth bg m, the Taylor
 * scatter (p.ntaylor; adjoint as p.adjoint_mode) and the depth step (p.prop),
 * added into the next depth; the adjoint runs upwards.  As the reference,
 * the forward clears the first output row whatever add says, and so does the
 * compat adjoint with the last row (LinOneWay.cpp:64-65); the exact adjoint
 * is the transpose.  in and out must differ. */
int wemop_lindown(wemop_handle* h, const void* bg, float freq, int adj, const void* in,
                  void* out, int add);

/* Element-wise operators of py_wem_ops (no handle). */
/* IC (ic.cpp:5-45): out (+)= bg in, adjoint conj(bg) in, over n values */
int wem_ic(const void* bg, int n, int adj, const void* in, void* out, int add);
/* Phshift (Phshift_cmplx.cpp:8-113, phase_shift.ispc:2-32): rows of n
 * wavenumber samples (the k grid of a row of n points at spacing dx) times
 * the phase-shift factor of slowness s = s_re + i s_im at frequency freq over
 * dz, with p->eps and p->phase_law; the adjoint takes the conjugate factor. */
int wem_phshift(const wem_params* p, int n, float dx, float dz, float freq, float s_re,
                float s_im, int adj, const void* in, void* out, int nrow, int add);
/* Injection (Injection.h:19-65, Injection.cpp:8-33, 52-75; py_wem_ops.cpp:181-198):
 * npt points (iz[i], ix[i]) of a row set data [nz][nx] (complex), each
 * spread over ix[i] + tap + [-ng, ng] with the cos^2 window, within the
 * row.  The model is complex [nt] (nshot = 0: every point takes
 * model[step]) or [nshot][npt][nt] (point i takes model[shot][i][step]).
 * Forward: data = (or += with add) the spread values; adjoint: model
 * (+)= the gathered values, the whole model cleared first unless add, as
 * the reference.  Depth indices outside [0, nz) are rejected (the
 * reference would write outside the rows); host or device pointers. */
int wem_inject(const int* iz, const int* ix, int npt, int ng, int tap, int nx, int nz, int nt, int nshot,
               int step, int shot, int adj, void* model, void* data, int add);
/* Reflect (Reflect.h:12-48) of the grid (slow2, rho) [nz][nx]: out = r in,
 * adjoint conj(r) in; assigned, as the reference's (no add). */
int wem_reflect(const void* slow2, const void* rho, int nx, int nz, int adj, const void* in,
                void* out);
/* dReflect (dReflect.h:11-84) at (slow2, rho) [nz][nx]: forward data (+)=
 * dR(dslow2, drho), adjoint (dslow2, drho) (+)= dR^H data. */
int wem_dreflect(const void* slow2, const void* rho, int nx, int nz, int adj, void* dslow2,
                 void* drho, void* data, int add);

/* One SSF/PSPI depth step that allocates no memory (no counterpart in the
 * reference).  It exists for callers that cannot call cudaMalloc while they
 * run: code that owns all device memory up front (a fixed arena or memory
 * pool, a real-time loop that must not touch the allocator) or whose
 * allocator is unavailable at that point.  Unlike wemop_onestep it needs no
 * handle: the caller passes the depth's inputs and the output, all in
 * device memory, and the per-call tables live in a 1 MiB device array that
 * the library holds on every GPU that loads it, until the process exits.
 *   slow_row  padded slowness^2 of the depth, complex [nxg]
 *   sref      reference slownesses of the depth, complex [nref]
 *   refidx    reference of each point [nxg] in [-1, nref) (-1: none),
 *             e.g. one row of wemop_refsampler's table; any other entry
 *             counts as -1 (the point gets no reference)
 *   in, out   complex [nrow][nxg]; adj and add as wemop_onestep
 * All five arrays must be memory of the current device (or managed).
 * Limits: N = nxg + 2 tap <= 4096 and nref <= 16 (WEM_EINVAL otherwise).
 * Every call reuses the same array, so calls that overlap on the GPU race:
 * serialise them.  The first call on a device looks the array up with
 * cudaGetSymbolAddress: make it before any stream capture (and the first
 * call after the device's context was reset, which looks it up again).
 * The work is queued on `stream` (a cudaStream_t, NULL for the default
 * stream) and the call returns without waiting for it. */
int wemop_onestep_noalloc(const wem_params* p, const void* slow_row, const void* sref,
                          const signed char* refidx, int nxg, float freq, int adj,
                          const void* in, void* out, int nrow, int add, void* stream);

/* ------------------------------------------- model-space interpolation
 * Coarse-to-fine interpolation of a 2D complex model, the preconditioner of
 * the FWI driver (scripts/fwi.py:45-68):
 *   data[i2][i1] = sum_j2 sum_j1 F2[i2][j2] F1[i1][j1] model[j2][j1],
 * model complex [nm2][nm1] (coarse), data complex [nd2][nd1] (fine), axis 1
 * fast.  The separable filters depend on the sampling intervals only (the
 * axes' origins are not used, as in the reference).  Pointers may be host
 * or device memory; add as above.
 *
 * lanczos2d_create: LanczosInterpolation2D
 *   (operator/src/LanczosInterpolation2D.h:14-125; Operator.py:436-445);
 *   a[0], a[1] = half widths in coarse samples along axes 1 and 2.
 * spline2d_create: Spline2D (operator/src/Spline2D.h:14-130;
 *   Operator.py:447-478), the cubic of parameters (a, b); its adjoint then
 *   copies the model's edge columns and rows from their neighbours
 *   (Spline2D.h:84-92), so it is not the transpose at the edges.
 * Both need at least 2 coarse samples per axis and positive intervals. */
typedef struct interp2d_handle interp2d_handle;

/* replaces pyOp.LanczosInterpolation2D(model, data, a) (operator/src/python/pyOp.cpp:55-64) */
int lanczos2d_create(int nm1, float dm1, int nm2, float dm2, int nd1, float dd1, int nd2, float dd2,
                     const float* a, interp2d_handle** out);
/* replaces pyOp.Spline2D(model, data, a, b) (operator/src/python/pyOp.cpp:66-75) */
int spline2d_create(int nm1, float dm1, int nm2, float dm2, int nd1, float dd1, int nd2, float dd2,
                    float a, float b, interp2d_handle** out);
void interp2d_destroy(interp2d_handle* h);
int interp2d_forward(interp2d_handle* h, const void* model, void* data, int add);
int interp2d_adjoint(interp2d_handle* h, void* model, const void* data, int add);

#ifdef __cplusplus
}
#endif

#endif /* WEMGPU_H */
