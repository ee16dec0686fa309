// Dispatch of the warp-per-row pass kernels (kernels_w.cuh) by row length.
#include "kernels.h"

namespace wg {

template <int E>
void launch_wem_w(const DevCtx& c, const Group* g, int ng, float2* store, float2* bins, cudaStream_t st);
template <int E>
void launch_fwd_w(const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm, float2* sA,
                  float2* sB, float2* bins, cudaStream_t st);
template <int E>
void launch_adj_w(const DevCtx& c, const Group* g, int ng, float2* sBG, float2* sT, float2* sG, float2* bins,
                  float2* ir, float2* is, int compat, cudaStream_t st);
template <int E>
bool adj_reuse_w(const DevCtx& c, int compat);
template <int E>
bool adj_split_w(const DevCtx& c);
template <int E>
size_t smem_w_e(const DevCtx& c, bool slots);
template <int E>
int adj_rows_w(const DevCtx& c);
template <int E>
int wem_rows_w(const DevCtx& c);

template <int E>
static int rows_e(const DevCtx& c, int which) {
  if (which == 0) return wem_rows_w<E>(c);
  if (which == 2) return adj_rows_w<E>(c);
  return 8;
}

int warp_rows_per_group(const DevCtx& c, int which) {
  switch (c.N / 32) {
    case 8: return rows_e<8>(c, which);
    case 12: return rows_e<12>(c, which);
    case 16: return rows_e<16>(c, which);
    case 24: return rows_e<24>(c, which);
    case 32: return rows_e<32>(c, which);
    default: return 8;
  }
}

bool warp_path_supported(const DevCtx& c) {
  if (c.N % 32 || c.ntaylor > 1) return false;
  int E = c.N / 32;
  return E == 8 || E == 12 || E == 16 || E == 24 || E == 32;
}

size_t warp_smem_bytes(const DevCtx& c, int which) {
  switch (c.N / 32) {
    case 8: return smem_w_e<8>(c, which == 2);
    case 12: return smem_w_e<12>(c, which == 2);
    case 16: return smem_w_e<16>(c, which == 2);
    case 24: return smem_w_e<24>(c, which == 2);
    case 32: return smem_w_e<32>(c, which == 2);
    default: return 0;
  }
}

template <int E>
static void launch_e(int which, const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm,
                     float2* s1, float2* s2, float2* s3, float2* bins, float2* ir, float2* is, int compat,
                     cudaStream_t st) {
  if (which == 0) launch_wem_w<E>(c, g, ng, s1, bins, st);
  else if (which == 1) launch_fwd_w<E>(c, g, ng, dm, drm, s1, s2, bins, st);
  else launch_adj_w<E>(c, g, ng, s1, s2, s3, bins, ir, is, compat, st);
}

void launch_pass_warp(int which, const DevCtx& c, const Group* g, int ng, const float2* dm, const float2* drm,
                      float2* s1, float2* s2, float2* s3, float2* bins, float2* ir, float2* is, int compat,
                      cudaStream_t st) {
  switch (c.N / 32) {
    case 8: launch_e<8>(which, c, g, ng, dm, drm, s1, s2, s3, bins, ir, is, compat, st); break;
    case 12: launch_e<12>(which, c, g, ng, dm, drm, s1, s2, s3, bins, ir, is, compat, st); break;
    case 16: launch_e<16>(which, c, g, ng, dm, drm, s1, s2, s3, bins, ir, is, compat, st); break;
    case 24: launch_e<24>(which, c, g, ng, dm, drm, s1, s2, s3, bins, ir, is, compat, st); break;
    case 32: launch_e<32>(which, c, g, ng, dm, drm, s1, s2, s3, bins, ir, is, compat, st); break;
    default: break;
  }
}

template <int E>
void launch_grad_w(const DevCtx& c, const Group* g, int ng, const GradArgs& a, cudaStream_t st);
template <int E>
bool grad_fits_w(const DevCtx& c);

bool grad_warp_supported(const DevCtx& c) {
  if (!warp_path_supported(c)) return false;
  switch (c.N / 32) {
    case 8: return grad_fits_w<8>(c);
    case 12: return grad_fits_w<12>(c);
    case 16: return grad_fits_w<16>(c);
    case 24: return grad_fits_w<24>(c);
    case 32: return grad_fits_w<32>(c);
    default: return false;
  }
}

// rows per CTA of the gradient kernel (kRowsAdj2 of kernels_w.cuh)
int grad_rows_per_group() { return 8; }

void launch_grad_warp(const DevCtx& c, const Group* g, int ng, const GradArgs& a, cudaStream_t st) {
  switch (c.N / 32) {
    case 8: launch_grad_w<8>(c, g, ng, a, st); break;
    case 12: launch_grad_w<12>(c, g, ng, a, st); break;
    case 16: launch_grad_w<16>(c, g, ng, a, st); break;
    case 24: launch_grad_w<24>(c, g, ng, a, st); break;
    case 32: launch_grad_w<32>(c, g, ng, a, st); break;
    default: break;
  }
}

bool warp_adj_split(const DevCtx& c) {
  switch (c.N / 32) {
    case 8: return adj_split_w<8>(c);
    case 12: return adj_split_w<12>(c);
    case 16: return adj_split_w<16>(c);
    case 24: return adj_split_w<24>(c);
    case 32: return adj_split_w<32>(c);
    default: return false;
  }
}

bool warp_adj_reuse(const DevCtx& c, int compat) {
  switch (c.N / 32) {
    case 8: return adj_reuse_w<8>(c, compat);
    case 12: return adj_reuse_w<12>(c, compat);
    case 16: return adj_reuse_w<16>(c, compat);
    case 24: return adj_reuse_w<24>(c, compat);
    case 32: return adj_reuse_w<32>(c, compat);
    default: return false;
  }
}

}  // namespace wg
