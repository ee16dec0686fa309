// Device-side context and host launchers of the GB300 kernels.
//
// Work unit: a row = one (shot, frequency) wavefield of nxg complex values.
// Rows are batched in groups of up to G shots of one frequency; one CTA
// runs a group through every depth step of a pass with the rows resident in
// shared memory, so a depth step costs no grid-wide synchronisation and the
// per-(frequency, depth) tables are read once per group.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "fft_plan.h"

namespace wg {

constexpr int kThreads = 512;  // threads per CTA of every pass kernel

struct DevCtx {
  FftPlan plan;                 // length N = nxg + 2 tap
  int N, nxg, tap, pad, nz, nref, prop, ntaylor, nfreq, ext, ns, nr, ngs, ngr, nbin;
  int phase_law;                // WEM_PHASE_ISPC or WEM_PHASE_EXACT_KZ
  // Born variants (BornRefl, BornTomo of propagator/src/ext_born_refl.cpp,
  // ext_born_tomo.cpp) on the Born passes:
  int ext_model;                // perturbation rows and images per frequency, tables shared
  const float2* rcf;            // [F][nz][nxg] per-frequency reflectivity replacing rc, or null
  int no_fwd_record;            // the forward-scattered (down) field is not recorded
  int last_rule;                // compat last depth row: 0 per shot (BornFull), 1 only the last (f, s)
  int one_row;                  // every group holds one row: the warp kernels use one-row CTAs
  float2* bg_store;             // [rows][nz][nxg]: the WEM pass also stores its down field here, or null
  int adj_split;                // the Born adjoint's down sweep is kw_adj_down's, on the stored bg
  float dz, invN;
  const float2* tw;             // [N] exp(-2 pi i t/N)
  const float2* ph;             // [F][nz][nref][N] phase-shift factors (phase_shift.ispc)
  const float2* fac;            // SSF: [F][nz][nxg] taper * split-step / N; PSPI: null
  const float* taperN;          // [nxg] taper / N
  const signed char* ref;       // [M][nz][nxg] reference of each point, -1 none
  const float2* sc;             // [M][ntaylor+1][nz][nxg] Scatter coefficients
  const float2* rc;             // [M][nz][nxg] Reflect coefficients
  const float* kx;              // [N] k grid
  const float* omega;           // [F] 2 pi f
  const int* bin;               // [F] data bin of each frequency
  const float2* wave;           // [F] wavelet spectrum at bin[f]
  const int* sx;                // [ns] source x (unpadded grid index), or the points of sptr
  const int* sptr;              // [ns + 1] source points of each shot in sx, or null: one per shot
  const int* sz;                // [ns] source depth index
  const float* gs;              // [2 ngs + 1] source window
  const float* gr;              // [2 ngr + 1] receiver window
  const int* rptr;              // [nz + 1] receivers by depth (CSR over rid)
  const int* rid;               // receiver ids sorted by (depth, x)
  const int* rxs;               // x of rid[k] (sorted within a depth)
  // exact gradient of the modelling (kernels_wg.cuh)
  const float2* gam;            // [F][nz][N] -i dz ph / (2 kz), the phase factor's derivative
  const float2* sref;           // [M][nz][nref] reference slownesses
};

// group g: frequency f, first shot s0, row count n, first storage row
struct Group {
  int f, s0, n, row0;
};

// shared-memory bytes of each pass for G rows per group
size_t smem_wem(const DevCtx& c, int G);
size_t smem_born_fwd(const DevCtx& c, int G);
size_t smem_born_adj(const DevCtx& c, int G);
size_t smem_rows(const DevCtx& c, int G);
int max_smem_per_block();
// grid of a table builder whose CTAs stride over nrow table rows (gx CTAs
// across a row, `threads` per CTA): enough CTAs for two waves on every SM, so
// each CTA walks many rows instead of the SMs scheduling one CTA per row
dim3 table_grid(int gx, int nrow, int threads);
// counts the library's kernel launches (wem_launch_count)
void note_launch();
long long launch_count();

#ifdef __CUDACC__
// reflection row of depth z for frequency f
__device__ __forceinline__ const float2* rc_row(const DevCtx& c, int f, int z) {
  return c.rcf ? c.rcf + ((size_t)f * c.nz + z) * c.nxg : c.rc + ((size_t)(c.ext ? f : 0) * c.nz + z) * c.nxg;
}
// offset of the perturbation row (dm, dR(dm)) of depth z for frequency f
__device__ __forceinline__ size_t pert_off(const DevCtx& c, int f, int z) {
  return ((size_t)((c.ext || c.ext_model) ? f : 0) * c.nz + z) * c.nxg;
}
// the as-coded Born adjoint keeps, in the last depth row, the LinUp^H term of
// one row only (LinOneWay.cpp:64-65 zeroes that row on every LinDown^H call)
__device__ __forceinline__ bool keep_last_row(const DevCtx& c, int compat, int f, int s) {
  if (!compat) return true;
  if (c.last_rule == 1) return f == c.nfreq - 1 && s == c.ns - 1;
  return c.ext ? (s == c.ns - 1) : (f == c.nfreq - 1);
}
#endif

// ---- table builders
void launch_phase_tables(const DevCtx& c, const float2* sref /*[M][nz][nref]*/, float eps, float2* ph,
                         cudaStream_t st);
void launch_fac_tables(const DevCtx& c, const float2* q /*[M][nz][nxg]*/, float2* fac, cudaStream_t st);

// ---- passes (one CTA per group)
void launch_wem(const DevCtx& c, const Group* groups, int ngroups, int G, float2* store, float2* bins,
                cudaStream_t st);
void launch_born_fwd(const DevCtx& c, const Group* groups, int ngroups, int G, const float2* dm,
                     const float2* drm, float2* storeA, float2* storeB, float2* bins, cudaStream_t st);
// compat: 0 exact, 1 compat (Scatter order + last-row rule).  last_f/last_s:
// the frequency / shot whose LinUp term keeps the last depth row in compat mode
void launch_born_adj(const DevCtx& c, const Group* groups, int ngroups, int G, float2* storeBG, float2* storeT,
                     const float2* bins, float2* imgR, float2* imgS, int compat, cudaStream_t st);

// row-level operators over rows of one frequency index f
void launch_onestep(const DevCtx& c, int f, int z, int adj, const float2* in, float2* out, int nrow, int add,
                    int G, cudaStream_t st);
void launch_scatter(const DevCtx& c, int f, int z, int adj, int exact, const float2* in, float2* out, int nrow,
                    int add, int G, cudaStream_t st);
// whole-field Down/Up; recursive = model aliases data (in-place drivers)
void launch_oneway(const DevCtx& c, int f, int up, int adj, int recursive, const float2* in, float2* out,
                   int nrow, int add, int G, cudaStream_t st);

// ---- warp-per-row passes (kernels_w.cu), N = 32 E with E in {8,12,16,24,32}
bool warp_path_supported(const DevCtx& c);
// rows (shots) per CTA of a warp-path pass (which: 0 WEM, 1 Born forward, 2 Born adjoint)
int warp_rows_per_group(const DevCtx& c, int which);
size_t warp_smem_bytes(const DevCtx& c, int which);
// which: 0 WEM, 1 Born forward, 2 Born adjoint (arguments as the launchers above)
void launch_pass_warp(int which, const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm,
                      float2* s1, float2* s2, float2* s3, float2* bins, float2* ir, float2* is, int compat,
                      cudaStream_t st);
// the Born adjoint's warp kernel reuses step spectra in its scatters and
// then needs s3: [rows][nz][nxg] filtered spectra of the stored T
bool warp_adj_reuse(const DevCtx& c, int compat);
// the FWI gradient's Born adjoint can run its down sweep as kw_adj_down on
// the source field the modelling pass stored (c.bg_store, c.adj_split)
bool warp_adj_split(const DevCtx& c);

// exact gradient of the modelling (kernels_wg.cuh), two warps per row, one
// reference; storage per row: full (ck <= 1) bg, t [nz][nxg] and sw, sg
// [nz][N]; checkpoints (ck > 1) bg, t [(nz - 1)/ck + 1][nxg] and seg
// [(ck + 1)(2 nxg + 2 N) + N]; per group: il, ir [nz][nxg]; qs [2][rows][nz]
struct GradArgs {
  float2 *bg, *t, *sw, *sg, *seg, *il, *ir, *qs;
  const float2* bins;
  int ck, rows_total;
};
bool grad_warp_supported(const DevCtx& c);
int grad_rows_per_group();
void launch_grad_warp(const DevCtx& c, const Group* g, int ng, const GradArgs& a, cudaStream_t st);
// Gamma = -i dz ph / (2 kz) of every phase-table entry (one reference)
void launch_phase_grad_tables(const DevCtx& c, const float2* sref, float eps, float2* gam, cudaStream_t st);
// out[z] (+)= sum over rows r of qs[0][r][z] + qs[1][r][z], rows in order
void launch_qs_reduce(const float2* qs, int rows, int nz, int add, float2* out, cudaStream_t st);
// gradient of the modelling on the model grid [nz][nx] from the images IR,
// IL [nz][nxg] and the per-depth reference sums qsum [nz] (exact derivatives
// of Reflect, the split-step and reference terms; edge-extended padding
// summed back onto the edge columns)
void launch_exact_assemble(const DevCtx& c, int nx, float eps, const float2* sp, const float2* dp, const float2* IR,
                           const float2* IL, const float2* qsum, float2* gref, float2* g0, float2* g1, int add,
                           cudaStream_t st);

// ---- subsurface-offset extended reflectivity Born (kernels_off.cuh,
// offset.cu).  Every shot propagates on its own aperture: model columns
// [x0, x0 + w) edge-padded by pad (nxg = w + 2 pad) and zero-padded by tap
// before and N - nxg - tap after it to a row of N = 32 E points.  A CTA holds
// up to kOffRows frequencies of one shot.  Per-shot tables are concatenated;
// rows (shot, frequency) are ordered by row length, then shot, then
// frequency, and each row has its own phase and split-step tables.
constexpr int kOffRows = 8;
struct OffCtx {
  int nz, nx, pad, prop, phase_law, nh, nfreq, ns, nr, ngs, ngr;
  float dz, eps;
  const float2* tw;        // [N] exp(-2 pi i t / N) of this launch's row length
  const float* kx;         // [N] k grid of this launch's row length
  const float* omega;      // [F] 2 pi f
  const float2* wave;      // [F] wavelet spectrum at the propagated bins
  const int* x0;           // [ns] first model column of the aperture
  const int* w;            // [ns] aperture width
  const int* tap;          // [ns] zero pad before the padded aperture in the row
  const long long* toff;   // [ns] offset of the shot's [nz][nxg] tables
  const float* taperN;     // [sum nxg] taper / N of each shot
  const int* tpo;          // [ns] offset of the shot's taper
  const float2* q;         // [sum nz nxg] split-step exponent (s - s_ref)/sqrt(s_ref);
                           // (0, kOffNoRef) where the point has no reference
  const float2* sref;      // [ns][nz] reference slowness
  const int* sx;           // source points (model columns), sptr as DevCtx
  const int* sptr;
  const int* sz;           // [ns] source depth
  const float* gs;         // [2 ngs + 1]
  const float* gr;         // [2 ngr + 1]
  const int* rptr;         // [ns][nz + 1] receivers of shot s at depth z in rid/rxc
  const int* rid;          // receiver index in the data
  const int* rxc;          // receiver model column, ascending within a (shot, depth)
  const int* rowbase;      // [ns] row of (s, f = 0); rows of a shot are consecutive in f
  const int* rowshot;      // [rows] shot of each row
  const long long* roff;   // [rows] offset of each row's [nz][nxg] field and split-step table
  const long long* poff;   // [rows] offset of each row's [nz][N] phase table
  const float2* tph;       // phase-shift factors of every row [nz][N] (phase_factor)
  const float2* tfac;      // split-step factors x taper / N of every row [nz][nxg] (ssf_factor)
};
// imaginary part of q at points without a reference: the split-step factor
// exp(w dz Im q) underflows to zero
constexpr float kOffNoRef = -1e30f;
struct OffGroup {
  int s, f0, n, row0;
};
// the phase and split-step tables of the rows [row0, row0 + nrows), all of
// row length N = 32 E (c.kx that length's k grid)
void launch_off_tables(const OffCtx& c, int row0, int nrows, int N, cudaStream_t st);
// row lengths of the warp kernels: N = 32 E, E in {8, 12, 16, 24, 32}
int off_row_length(int min_n);  // smallest such N >= min_n, or 0
size_t off_smem_bytes(int E, int nxg_max);
// mode 0: down sweep of the source field, stored; 1: up sweep of the stored
// source rows, recorded into bins [ns][nr][F]; 2: adjoint of the up sweep of
// the recorded bins, stored
void launch_off_sweep(int mode, int E, const OffCtx& c, const OffGroup* g, int ng, int nxg_max, float2* store,
                      float2* bins, cudaStream_t st);
// scattered source sc(x) = sum_l r_l(x - l) bg(x - 2l) of every row of the
// shots (rows laid out as the stores), model [nh][nz][nx]
void launch_off_source(const OffCtx& c, const float2* model, const float2* bg, float2* sc, int nxg_max,
                       cudaStream_t st);
// img [nh][nz][nx] (+)= sum over rows of conj(bg(x - l)) a(x + l)
void launch_off_image(const OffCtx& c, const float2* bg, const float2* a, float2* img, int add, cudaStream_t st);
// padded apertures [sum nz nxg] of the slowness [nz][nx] (edge-extended,
// each aperture on its own: operator/src/Pad.h:77-96)
void launch_off_crop(const OffCtx& c, const float2* s2, int nxg_max, float2* sp, cudaStream_t st);
// q of every point of the apertures from the padded slowness, the reference
// slownesses [ns][nz] and the partition [sum nz nxg] (ssf: the split step's
// (s - s_ref)/sqrt(s_ref), SplitStep.cpp:12-13; else 0)
void launch_off_q(const OffCtx& c, const float2* sp, const signed char* ref, int ssf, int nxg_max, float2* q,
                  cudaStream_t st);

// ---- 3D one-way operators (k3d.cu).  A (shot, frequency) row is a plane of
// Ny x Nx FFT points (Nx = 32 Ex; Ny = 32 Ey or 1) holding the padded model
// slice nyg x nxg at offset (tapy, tapx).  A depth step is two batched
// passes over all rows: the column pass (transforms along y, the phase shift
// per reference) and the row pass (transforms along x and every point
// operation).  Rows r = f ns + s.
struct Ctx3 {
  int Nx, Ny, nxg, nyg, tapx, tapy, pad, pady, nx, ny, nz, nref, prop, ns, nr, nfreq, ngs, ngr, rows;
  int Qx, Qy;              // quadrant of the phase tables: Nx / 2 x max(Ny / 2, 1)
  float dz;
  const float2* twx;       // [Nx] exp(-2 pi i t / Nx)
  const float2* twy;       // [Ny]
  const float* taper;      // [nyg][nxg] taper_x taper_y / (Nx Ny)
  const float2* ph;        // [F][nz][nref][Qy][Qx] phase-shift factors by |kx|, |ky|
  const float2* q;         // [nz][nyg][nxg] split-step exponent (SSF), null for PSPI
  const signed char* ref;  // [nz][nyg][nxg] reference of each point, -1 none
  const float2* rc;        // [nz][nyg][nxg] Reflect coefficients
  const float* omega;      // [F]
  const float2* wave;      // [F]
  const int* sx;           // [ns] source column, row, depth (model grid)
  const int* sy;
  const int* sz;
  const float* gs;         // [2 ngs + 1] spreading along x
  const float* gr;         // [2 ngr + 1]
  const int* rptr;         // [nz * nyg + 1] receivers by (depth, padded line) in rid / rxs
  const int* rid;
  const int* rxs;          // receiver model column, ascending within a line
};
// per-launch arguments of the row pass; planes of stored fields are
// [rows][nyg][nxg]
struct Pass3 {
  int z;                   // depth of the field this pass produces (forward) or reads (adjoint)
  int zt;                  // depth of the split-step tables applied in this pass (-1 none)
  int init;                // 0: from the transform input, 1: zero, 2: load `load`
  int src;                 // inject the source at depth z
  int rec_in;              // add the receivers' data of depth z (adjoint of the record)
  int record;              // record the field at the receivers of depth z
  int last;                // no transform output
  const float2* load;      // init 2: the field
  float2* store;           // the field (or R[z] x field with store_rw) out
  int store_rw;
  const float2* add;       // field += add (add_rw: R[z] x add; add_refl: refl[z] x add)
  int add_rw;
  const float2* refl;      // [nz][ny][nx] reflectivity of add_refl (model grid)
  float2* spatial;         // the field out (imaging)
  const float2* tin;       // transform input planes: forward nref x [rows][Ny][Nx], adjoint [rows][Ny][Nx]
  float2* tout;            // transform output planes: forward [rows][Ny][Nx], adjoint nref x [rows][Ny][Nx]
  float2* bins;            // [ns][nr][F]
};
bool k3_supported(int Nx, int Ny);
// row pass (adj: the adjoint step's order: inverse transform, point
// operations, per-reference split step and forward transform)
void launch_k3_rows(const Ctx3& c, const Pass3& a, int adj, cudaStream_t st);
// column pass of the step at depth z: forward S -> T_j (nref planes),
// adjoint T_j -> S
void launch_k3_cols(const Ctx3& c, int z, int adj, const float2* in, float2* out, cudaStream_t st);
// image[z][y][x] (+)= sum over rows (in order) conj(bg) a at depth z
void launch_k3_image(const Ctx3& c, int z, const float2* bg, const float2* a, float2* img, int add, cudaStream_t st);
// quadrant phase tables from the reference slownesses [nz][nref] and the
// k grids
void launch_k3_phase(const Ctx3& c, const float2* sref, const float* kx, const float* ky, float eps, int law,
                     float2* ph, cudaStream_t st);
// edge-extended padding of [M][nz][ny][nx] to [M][nz][nyg][nxg]
void launch_pad3(const float2* in, float2* out, int nz, int ny, int nx, int pady, int pad, cudaStream_t st);

// ---- background tables on the device (tables.cu)
void launch_pad_edge(const float2* in, float2* out, int M, int nz, int nx, int pad, cudaStream_t st);
// reference slownesses [M][nz][nref]; bad (may be null): atomicMin of the
// flat index of any entry whose real part is not > 0
void launch_sref(const float2* sp, float2* sref, int M, int nz, int nxg, int nref, int* bad, cudaStream_t st);
// RefSampler partition (as coded, or nearest): reference index [M][nz][nxg]
// of every point from the padded slowness and the reference slownesses;
// scratch holds refs_scratch_floats(M, nz, nref) floats
size_t refs_scratch_floats(int M, int nz, int nref);
void launch_refsampler(int nearest, const float2* sp, const float2* sref, int M, int nz, int nxg, int nref,
                       float* scratch, signed char* ref, cudaStream_t st);
// q (SSF split step, may be null), rc, and for the Born operators sc and the
// dReflect pairs (null to skip) of every padded point
// sp_refl: the slowness of the Reflect/dReflect coefficients when it differs
// from sp (conformal maps scale sp by the Jacobian after Reflect is built);
// null = sp
void launch_point_tables(int M, int nz, int nxg, int nref, int ntaylor, float eps, const float2* sp,
                         const float2* sp_refl, const float2* dp, const float2* sref, const signed char* ref,
                         float2* q, float2* rc, float2* sc, float2* a0, float2* b0, float2* a1, float2* b1,
                         cudaStream_t st);
// conformal maps: out[i] = in[idx[i]] (0 where idx < 0); add < 0 overwrites,
// 0/1 as the operators' add
void launch_cmap_gather(const float2* in, const int* idx, float2* out, int n, int add, cudaStream_t st);
// sp[k] *= js, *= jl[k] (jl may be null), twice, for k < n
void launch_cmap_jacobian(float2* sp, int n, float js, const float* jl, cudaStream_t st);

// ---- helpers
void launch_pad_model(const float2* in, float2* out, int M, int nz, int nx, int pad, cudaStream_t st);
void launch_drefl_fwd(const DevCtx& c, int M, const float2* a0, const float2* b0, const float2* a1,
                      const float2* b1, const float2* dm0, const float2* dm1, float2* out, cudaStream_t st);
void launch_reduce_images(const float2* parts, const int* slice_beg, int M, size_t plane, float2* out,
                          cudaStream_t st);
void launch_grad_assemble(const DevCtx& c, int M, const float2* a0, const float2* b0, const float2* a1,
                          const float2* b1, const float2* IR, const float2* IS, float2* g0, float2* g1, int nx,
                          int add, cudaStream_t st);
// ---- time <-> frequency (timefreq.cu): real traces [ntr][nt] <-> compact
// bins [ntr][nf] at the consecutive FFT bins b0 .. b0 + nf - 1 of length n
struct TfStage {
  int R, L, nb, twoff, ld;   // radix, product of the earlier radices, n / R, offset in tws, padded row length
  unsigned mag_nb, mag_L;    // ceil(2^32 / nb), ceil(2^32 / L) (unused when 1)
  float2 w7[7];              // exp(-2 pi i m / 7) (radix 7)
};
struct TimeFreq {
  FftPlan plan;              // radices of n = nt + tpad
  TfStage st[kMaxStages];
  const float2* tws;         // per-stage twiddles [(R - 1) L] in stage order
  int tw_len;
  const float2* wn;          // [n] exp(-2 pi i j / n) (the restricted DFT)
  int n, nt, nf, b0;
  int fft;                   // every prime factor of n is <= 7
  float sc;                  // 1/sqrt(n)
};
// launch shape: the FFT path with R traces per CTA, or the restricted DFT
// (use_fft 0); ok 0 when the DFT's traces do not fit in shared memory
struct TfShape {
  int R, grid, use_fft, ok;
  size_t smem;
};
TfShape timefreq_shape(const TimeFreq& t, int ntr);
// mode 0: time (+)= Re IFFT(bins) sc (add), 1: bins = FFT(time) sc,
// 2: bins <- FFT(Re IFFT(bins) sc - obs) sc and part[grid] the per-CTA sums
// of the squared residual (double)
void launch_timefreq(int mode, const TimeFreq& t, const TfShape& s, float2* bins, float* time, const float* obs,
                     int ntr, int add, double* part, cudaStream_t st);
// out[0] = 1/2 sum part[0..n) in a fixed order
void launch_half_sum(const double* part, int n, double* out, cudaStream_t st);
// caller bins [nrows][ldu] <-> compact propagated bins [nrows][nf] (window at off)
void launch_bin_window(const float2* src, float2* dst, int nrows, int ldu, int nf, int off, int to_user, int add,
                       cudaStream_t st);
void launch_copy_rows(const float2* src, int lds, float2* dst, int ldd, int nrows, int ncopy, int add,
                      cudaStream_t st);
void launch_scale_add(float2* y, const float2* x, size_t n, cudaStream_t st);

// ---- element-wise operators of the row-level API (rowops.cu)
// out[r][k] = f[k] in[r][k] (conj(f) with conj), added with add
void launch_diag_rows(const float2* in, const float2* f, float2* out, int n, int nrow, int conj, int add,
                      cudaStream_t st);
// Injection (Injection.cpp:8-33, 52-75) between point values m_i =
// model[off0 + i stride] (stride 0: one sample for every point) and a
// [nz][nx] row set, cos^2 window g[2 ng + 1], points (iz[i], ix[i] + tap);
// forward assigns or adds data, the adjoint adds into model
void launch_inject(const int* iz, const int* ix, int npt, const float* g, int ng, int tap, int nx, int nz, int adj,
                   float2* model, size_t off0, size_t stride, float2* data, int add, cudaStream_t st);
// SplitStep at the points loc[0..nloc) of rows of nx points (srow: the
// slowness^2 row of the depth); the other points are not touched
void launch_splitstep(const float2* srow, const int* loc, int nloc, int nx, int nrow, double wdz, double sr,
                      double si, int adj, const float2* in, float2* out, cudaStream_t st);

}  // namespace wg
