// Adjoints (transposes) of the transforms and of soft thresholding, and the
// gradients of the cross-validation and SURE losses with respect to one soft
// threshold per level.  No counterpart in the reference: this serves
// gradient-based threshold tuning.
//
// Operators (periodic, as computed by dwt.cu / modwt.cu):
//  * DWT: the inverse applies exactly the transposed taps of the forward, so
//    adjoint(forward) = inverse and adjoint(inverse) = forward.
//  * TO-MODWT level: forward S = H_s X, D = G_s X; inverse X = (H_s^T S +
//    G_s^T D) / 2.  So adjoint(inverse level) = forward level / 2, and the
//    adjoint of the whole inverse is the forward transform with block l scaled
//    by 2^-(l+1) (intermediate s blocks receive no cotangent: the inverse does
//    not read them).  adjoint(forward level) = 2 x inverse level, and because
//    every s_l is also an output, the adjoint of the whole forward adds the
//    s_l cotangent before descending a level.
//  * Soft threshold eta(c) = sign(c) (|c| - t) for |c| >= t, else 0
//    (thresh.cpp:142-157): d eta / dc = 1{|c| >= t}, d eta / dt =
//    -sign(c) 1{|c| >= t}.
#include <math.h>

#include <algorithm>
#include <vector>

#include "wc_common.cuh"
#include "wc_dd.cuh"

namespace wc {

template <class T>
int threshold_to(const T* in, T* out, int64_t n, int J, int ttype, double t, int hardness,
                 int minl, int maxl, int copy_scaling, cudaStream_t s);

namespace {

constexpr int kThreads = 256;
constexpr int kMaxLevels = 32;

unsigned grid_for(int64_t n) {
  int64_t blocks = (n + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 8));
}

struct LevelVec {
  double v[kMaxLevels];
};

__device__ __forceinline__ int dwt_level(int64_t i) { return __ffsll((long long)i) - 1; }

// Soft thresholds per level (lambda[l]) on a DWT (in -> out, interleaved) or
// a time-ordered MODWT (detail blocks); levels outside [minl, maxl] and
// scaling coefficients are copied.
__global__ void soft_levels_kernel(const double* __restrict__ in, double* __restrict__ out,
                                   int64_t n, int J, int ttype, LevelVec lambda, int minl,
                                   int maxl) {
  const int64_t total = (ttype == 0) ? n : 2 * n * (int64_t)J;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    int l;
    bool det;
    if (ttype == 0) {
      l = (e == 0) ? J : dwt_level(e);
      det = l < J;
    } else {
      l = (int)(e / (2 * n));
      det = (e - (int64_t)l * 2 * n) >= n;
    }
    double c = in[e];
    if (det && l >= minl && l <= maxl) {
      const double t = lambda.v[l];
      c = (fabs(c) < t) ? 0.0 : __dmul_rn((c < 0) ? -1.0 : 1.0, __dsub_rn(fabs(c), t));
    }
    out[e] = c;
  }
}

// Per-level sums g[l] = sum_i gc_i * (-sign(c_i)) * 1{|c_i| >= lambda_l} over
// the thresholded detail coefficients; also gcoef = gc * 1{|c| >= lambda}.
__global__ void soft_adjoint_kernel(const double* __restrict__ c, const double* __restrict__ gc,
                                    double* __restrict__ gcoef, double* __restrict__ glam,
                                    int64_t n, int J, int ttype, LevelVec lambda, int minl,
                                    int maxl) {
  __shared__ double acc[kMaxLevels];
  for (int i = threadIdx.x; i < kMaxLevels; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const int64_t total = (ttype == 0) ? n : 2 * n * (int64_t)J;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    int l;
    bool det;
    if (ttype == 0) {
      l = (e == 0) ? J : dwt_level(e);
      det = l < J;
    } else {
      l = (int)(e / (2 * n));
      det = (e - (int64_t)l * 2 * n) >= n;
    }
    const double g = gc[e];
    if (det && l >= minl && l <= maxl) {
      const double ce = c[e];
      const bool keep = !(fabs(ce) < lambda.v[l]);
      if (gcoef) gcoef[e] = keep ? g : 0.0;
      if (keep && g != 0.0) atomicAdd(&acc[l], (ce < 0) ? g : -g);
    } else if (gcoef) {
      gcoef[e] = g;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < J && i < kMaxLevels; i += blockDim.x)
    if (acc[i] != 0.0) atomicAdd(&glam[i], acc[i]);
}

// Scales MODWT block b (0 .. 2J-1) by s_b: d blocks of level l by 2^-(l+1),
// the top s block by 2^-J, intermediate s blocks to zero.
__global__ void modwt_adj_scale_kernel(double* __restrict__ xm, int64_t n, int J) {
  const int64_t total = 2 * n * (int64_t)J;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int b = (int)(e / n), l = b / 2;
    double sc;
    if (b & 1) sc = ldexp(1.0, -(l + 1));
    else sc = (l == J - 1) ? ldexp(1.0, -J) : 0.0;
    xm[e] = xm[e] * sc;
  }
}

// One level of the adjoint of the forward MODWT:
// out[i] = sum_k (h_k A[i - k s] + g_k Gd[i - k s]) (+ Gs[i] when Gs != null).
template <int F>
__global__ void modwt_adj_fwd_level(const double* __restrict__ A, const double* __restrict__ Gd,
                                    const double* __restrict__ Gs, double* __restrict__ out,
                                    int64_t n, int64_t skip) {
  constexpr int L = filter_len(F);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < L; k++) {
      const int64_t j = (i - (int64_t)k * skip) & (n - 1);
      acc = fma(tap_h(F, k), A[j], acc);
      acc = fma(tap_g(F, k), Gd[j], acc);
    }
    out[i] = Gs ? acc + Gs[i] : acc;
  }
}

// Cotangents of the CV loss (interp_mse, thresh.cpp:344-385) with respect to
// the two half-length reconstructions, and the terms of the loss:
//   a_j = yie_j - x[2j], b_j = yio_j - x[2j+1];  loss = 0.5 sum (a^2 + b^2)
//   d/dyo[k] = [k==0] a_0 + [k>=1] a_k/2 + [k<=lenh-2] a_{k+1}/2
//   d/dye[k] = [k<=lenh-2] b_k/2 + [k>=1] b_{k-1}/2 + [k==lenh-1] b_{lenh-1}
__device__ __forceinline__ void interp_ab(const double* ye, const double* yo, const double* x,
                                          int64_t lenh, int64_t j, double& a, double& b) {
  double yie, yio;
  if (j == 0) {
    yie = yo[0];
    yio = 0.5 * (ye[0] + ye[1]);
  } else if (j == lenh - 1) {
    yio = ye[lenh - 1];
    yie = 0.5 * (yo[j] + yo[j - 1]);
  } else {
    yio = 0.5 * (ye[j] + ye[j + 1]);
    yie = 0.5 * (yo[j] + yo[j - 1]);
  }
  a = yie - x[2 * j];
  b = yio - x[2 * j + 1];
}

__global__ void cv_adjoint_kernel(const double* __restrict__ ye, const double* __restrict__ yo,
                                  const double* __restrict__ x, int64_t lenh,
                                  double* __restrict__ gye, double* __restrict__ gyo,
                                  double* __restrict__ loss) {
  double part = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < lenh; k += stride) {
    double a, b;
    interp_ab(ye, yo, x, lenh, k, a, b);
    part += a * a + b * b;
    double go = (k == 0) ? a : 0.5 * a;
    double ge = (k == lenh - 1) ? b : 0.5 * b;
    if (k + 1 <= lenh - 1) {
      double a1, b1;
      interp_ab(ye, yo, x, lenh, k + 1, a1, b1);
      go += 0.5 * a1;
    }
    if (k >= 1) {
      double a0, b0;
      interp_ab(ye, yo, x, lenh, k - 1, a0, b0);
      if (k - 1 <= lenh - 2) ge += 0.5 * b0;
    }
    gyo[k] = go;
    gye[k] = ge;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, 0.5 * part);
}

}  // namespace
}  // namespace wc

namespace wc {

// Adjoint of the DWT: forward <-> inverse (exact transposes).
int dwt_adjoint(const void* gin, void* gout, int64_t n, int sense, int J, int F, int prec,
                cudaStream_t s) {
  return dwt(gin, gout, n, sense == 1 ? 0 : 1, J, F, prec, s);
}

namespace {

template <int F>
int modwt_adj_fwd(const double* gxmod, double* gx, int64_t n, int J, double* tmp0,
                  double* tmp1, cudaStream_t s) {
  const double* A = gxmod + (int64_t)2 * (J - 1) * n;
  for (int l = J - 1; l >= 0; l--) {
    double* out = (l == 0) ? gx : ((l & 1) ? tmp1 : tmp0);
    const double* Gs = (l >= 1) ? gxmod + (int64_t)2 * (l - 1) * n : nullptr;
    modwt_adj_fwd_level<F><<<grid_for(n), kThreads, 0, s>>>(
        A, gxmod + (int64_t)(2 * l + 1) * n, Gs, out, n, (int64_t)1 << l);
    WC_TRY(after_launch("modwt_adj_fwd_level"));
    A = out;
  }
  return WC_OK;
}

}  // namespace

// Adjoint of the time-ordered MODWT in FP64.  sense FWD: gxmod (cotangents of
// all 2J blocks) -> gx.  sense BWD: gx (cotangent of the reconstruction) ->
// gxmod (cotangents of s_J and d_1..d_J; zero for the other s blocks).
int modwt_adjoint(double* gx, double* gxmod, int64_t n, int sense, int J, int F,
                  cudaStream_t s) {
  if (sense == 0) {
    WC_TRY(modwt(gx, gxmod, n, 1, J, F, WC_F64_EXACT, s));
    modwt_adj_scale_kernel<<<grid_for(2 * n * J), kThreads, 0, s>>>(gxmod, n, J);
    return after_launch("modwt_adj_scale_kernel");
  }
  double* t0 = nullptr;
  double* t1 = nullptr;
  if (J > 1) {
    t0 = static_cast<double*>(workspace(kSlotModwt0, sizeof(double) * (size_t)n));
    t1 = static_cast<double*>(workspace(kSlotModwt1, sizeof(double) * (size_t)n));
    if (!t0 || !t1) return workspace_error();
  }
  switch (F) {
    case 1: return modwt_adj_fwd<1>(gxmod, gx, n, J, t0, t1, s);
    case 2: return modwt_adj_fwd<2>(gxmod, gx, n, J, t0, t1, s);
    case 3: return modwt_adj_fwd<3>(gxmod, gx, n, J, t0, t1, s);
    case 4: return modwt_adj_fwd<4>(gxmod, gx, n, J, t0, t1, s);
  }
  return fail(WC_ERR_ARG, "unknown filter %d", F);
}

int soft_levels(const double* in, double* out, int64_t n, int J, int ttype, const double* lam,
                int minl, int maxl, cudaStream_t s) {
  LevelVec lv{};
  for (int l = 0; l < J && l < kMaxLevels; l++) lv.v[l] = lam[l];
  const int64_t total = (ttype == 0) ? n : 2 * n * (int64_t)J;
  soft_levels_kernel<<<grid_for(total), kThreads, 0, s>>>(in, out, n, J, ttype, lv, minl, maxl);
  return after_launch("soft_levels_kernel");
}

// glam (device, J doubles) += per-level threshold gradient; gcoef optional.
int soft_adjoint(const double* c, const double* gc, double* gcoef, double* glam, int64_t n,
                 int J, int ttype, const double* lam, int minl, int maxl, cudaStream_t s) {
  LevelVec lv{};
  for (int l = 0; l < J && l < kMaxLevels; l++) lv.v[l] = lam[l];
  const int64_t total = (ttype == 0) ? n : 2 * n * (int64_t)J;
  soft_adjoint_kernel<<<grid_for(total), kThreads, 0, s>>>(c, gc, gcoef, glam, n, J, ttype, lv,
                                                          minl, maxl);
  return after_launch("soft_adjoint_kernel");
}

// ------------------------------------------------------------ losses -----
namespace {

// Accumulator layout (device, FP64): [0] loss sum, [1 + l] threshold gradient
// of level l, [1 + 32 + l] smoothed kept count of level l, [1 + 64 + l] its
// derivative with respect to lambda_l.
constexpr int kAccLoss = 0, kAccGrad = 1, kAccKept = 1 + kMaxLevels, kAccDKept = 1 + 2 * kMaxLevels;
constexpr int kAccLen = 1 + 3 * kMaxLevels;

__global__ void split_kernel(const double* __restrict__ x, int64_t h, double* __restrict__ e,
                             double* __restrict__ o) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < h; j += stride) {
    e[j] = x[2 * j];
    o[j] = x[2 * j + 1];
  }
}

// g = 2 (fh - y); acc += sum (fh - y)^2.
__global__ void residual_kernel(const double* __restrict__ fh, const double* __restrict__ y,
                                double* __restrict__ g, int64_t n, double* __restrict__ acc) {
  double part = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double r = fh[i] - y[i];
    part = fma(r, r, part);
    g[i] = 2.0 * r;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, part);
}

// Smoothed kept indicator of soft thresholding, Phi((|c| - lambda) / eps)
// with the logistic Phi (eps == 0: the indicator itself, derivative 0).
__device__ __forceinline__ void smooth_keep(double c, double t, double eps, double& phi,
                                            double& dphi) {
  if (eps > 0.0) {
    const double u = (fabs(c) - t) / eps;
    phi = 1.0 / (1.0 + exp(-u));
    dphi = -phi * (1.0 - phi) / eps;  // d phi / d lambda
  } else {
    phi = (fabs(c) < t) ? 0.0 : 1.0;
    dphi = 0.0;
  }
}

// Per-level sums of the smoothed kept indicator and of its lambda-derivative
// over the thresholded detail coefficients (the divergence term of SURE).
__global__ void sure_div_kernel(const double* __restrict__ c, int64_t n, int J, int ttype,
                                LevelVec lambda, int minl, int maxl, double eps,
                                double* __restrict__ acc) {
  __shared__ double sk[kMaxLevels], sd[kMaxLevels];
  for (int i = threadIdx.x; i < kMaxLevels; i += blockDim.x) sk[i] = sd[i] = 0.0;
  __syncthreads();
  const int64_t total = (ttype == 0) ? n : 2 * n * (int64_t)J;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    int l;
    bool det;
    if (ttype == 0) {
      l = (e == 0) ? J : dwt_level(e);
      det = l < J;
    } else {
      l = (int)(e / (2 * n));
      det = (e - (int64_t)l * 2 * n) >= n;
    }
    if (!det || l < minl || l > maxl) continue;
    double phi, dphi;
    smooth_keep(c[e], lambda.v[l], eps, phi, dphi);
    atomicAdd(&sk[l], phi);
    if (dphi != 0.0) atomicAdd(&sd[l], dphi);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < J && i < kMaxLevels; i += blockDim.x) {
    if (sk[i] != 0.0) atomicAdd(&acc[kAccKept + i], sk[i]);
    if (sd[i] != 0.0) atomicAdd(&acc[kAccDKept + i], sd[i]);
  }
}

}  // namespace

// Applies the transform (FWD: x -> c) in FP64.
static int fwd_transform(const double* x, double* c, int64_t n, int J, int F, int ttype,
                         cudaStream_t s) {
  if (ttype == 0) return dwt(x, c, n, 1, J, F, WC_F64_EXACT, s);
  return modwt(const_cast<double*>(x), c, n, 1, J, F, WC_F64_EXACT, s);
}

// Inverse (c -> x) in FP64; c is not modified.
static int inv_transform(const double* c, double* x, int64_t n, int J, int F, int ttype,
                         cudaStream_t s) {
  if (ttype == 0) return dwt(c, x, n, 0, J, F, WC_F64_EXACT, s);
  return modwt(x, const_cast<double*>(c), n, 0, J, F, WC_F64_EXACT, s);
}

// Cotangent of the coefficients from the cotangent of an inverse transform's
// output (adjoint of the inverse).
static int inv_adjoint(double* gx, double* gc, int64_t n, int J, int F, int ttype,
                       cudaStream_t s) {
  if (ttype == 0) return dwt_adjoint(gx, gc, n, 0, J, F, WC_F64_EXACT, s);
  return modwt_adjoint(gx, gc, n, 0, J, F, s);
}

static int64_t coef_len(int64_t n, int J, int ttype) { return ttype == 0 ? n : 2 * n * (int64_t)J; }

// Per-level trace weight of the synthesis-analysis product (kappa_l) and the
// number of level-l detail coefficients: DWT is orthonormal (kappa 1, n/2^(l+1)
// coefficients); the TO-MODWT inverse scales level l by 2^-(l+1) over n
// coefficients of a unit-norm equivalent filter.
static void level_weights(int64_t n, int l, int ttype, double* kappa, double* count) {
  if (ttype == 0) {
    *kappa = 1.0;
    *count = (double)(n >> (l + 1));
  } else {
    *kappa = ldexp(1.0, -(l + 1));
    *count = (double)n;
  }
}

int sure_loss_grad(const double* y, int64_t n, int J, int F, int ttype, const double* lam,
                   int minl, int maxl, double sigma, double eps, double* loss, double* grad,
                   double* sigma_out, cudaStream_t s) {
  const int64_t nc = coef_len(n, J, ttype);
  const size_t bytes = sizeof(double) * (size_t)(2 * nc + 2 * n + kAccLen);
  double* base = static_cast<double*>(workspace(kSlotAdjoint, bytes));
  if (!base) return workspace_error();
  double* c = base;
  double* ch = c + nc;
  double* fh = ch + nc;
  double* g = fh + n;
  double* acc = g + n;
  WC_TRY(fwd_transform(y, c, n, J, F, ttype, s));
  if (!(sigma > 0.0)) {
    // Noise level from the finest details: MAD of the level-0 detail block.
    SelectSource src{ttype == 0 ? nullptr : c + n, n, n, 1};
    if (ttype == 0) {
      double* d0 = ch;  // gather the level-0 DWT details (odd indices)
      split_kernel<<<grid_for(n / 2), kThreads, 0, s>>>(c, n / 2, fh, d0);
      WC_TRY(after_launch("split_kernel"));
      src = SelectSource{d0, n / 2, n / 2, 1};
    }
    double med = 0.0;
    WC_TRY(median_mad(src, src.seg_len, s, &med, &sigma));
  }
  if (sigma_out) *sigma_out = sigma;
  WC_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * kAccLen, s));
  WC_TRY(soft_levels(c, ch, n, J, ttype, lam, minl, maxl, s));
  WC_TRY(inv_transform(ch, fh, n, J, F, ttype, s));
  residual_kernel<<<grid_for(n), kThreads, 0, s>>>(fh, y, g, n, acc + kAccLoss);
  WC_TRY(after_launch("residual_kernel"));
  WC_TRY(inv_adjoint(g, ch, n, J, F, ttype, s));
  WC_TRY(soft_adjoint(c, ch, nullptr, acc + kAccGrad, n, J, ttype, lam, minl, maxl, s));
  LevelVec lv{};
  for (int l = 0; l < J; l++) lv.v[l] = lam[l];
  sure_div_kernel<<<grid_for(nc), kThreads, 0, s>>>(c, n, J, ttype, lv, minl, maxl, eps, acc);
  WC_TRY(after_launch("sure_div_kernel"));
  double h[kAccLen];
  WC_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
  WC_TRY(take_status(s));
  // SURE = ||fh - y||^2 - n sigma^2 + 2 sigma^2 div, div = n - sum over
  // thresholded levels of kappa_l (count_l - smoothed kept_l).
  const double s2 = sigma * sigma;
  double div = (double)n;
  for (int l = 0; l < J; l++) {
    double kappa, count;
    level_weights(n, l, ttype, &kappa, &count);
    const bool thr = l >= minl && l <= maxl;
    if (thr) div -= kappa * (count - h[kAccKept + l]);
    grad[l] = thr ? h[kAccGrad + l] + 2.0 * s2 * kappa * h[kAccDKept + l] : 0.0;
  }
  *loss = h[kAccLoss] - (double)n * s2 + 2.0 * s2 * div;
  return WC_OK;
}

// Two-fold cross-validation loss of per-level soft thresholds (the loss of
// interp_mse, thresh.cpp:344-385, on the even/odd halves transformed with
// J - 1 levels, half levels [minl, min(maxl, J - 2)] thresholded by lam[l]).
int cv_loss_grad(const double* x, int64_t n, int J, int F, int ttype, const double* lam,
                 int minl, int maxl, double* loss, double* grad, cudaStream_t s) {
  const int64_t h = n / 2;
  const int Jh = J - 1;
  const int maxh = std::min(maxl, Jh - 1);
  const int64_t nc = coef_len(h, Jh, ttype);
  const size_t bytes = sizeof(double) * (size_t)(3 * nc + 6 * h + kAccLen);
  double* base = static_cast<double*>(workspace(kSlotAdjoint, bytes));
  if (!base) return workspace_error();
  double* ce = base;
  double* co = ce + nc;
  double* ch = co + nc;
  double* xe = ch + nc;
  double* xo = xe + h;
  double* ye = xo + h;
  double* yo = ye + h;
  double* gye = yo + h;
  double* gyo = gye + h;
  double* acc = gyo + h;
  WC_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * kAccLen, s));
  split_kernel<<<grid_for(h), kThreads, 0, s>>>(x, h, xe, xo);
  WC_TRY(after_launch("split_kernel"));
  WC_TRY(fwd_transform(xe, ce, h, Jh, F, ttype, s));
  WC_TRY(fwd_transform(xo, co, h, Jh, F, ttype, s));
  WC_TRY(soft_levels(ce, ch, h, Jh, ttype, lam, minl, maxh, s));
  WC_TRY(inv_transform(ch, ye, h, Jh, F, ttype, s));
  WC_TRY(soft_levels(co, ch, h, Jh, ttype, lam, minl, maxh, s));
  WC_TRY(inv_transform(ch, yo, h, Jh, F, ttype, s));
  cv_adjoint_kernel<<<grid_for(h), kThreads, 0, s>>>(ye, yo, x, h, gye, gyo, acc + kAccLoss);
  WC_TRY(after_launch("cv_adjoint_kernel"));
  WC_TRY(inv_adjoint(gye, ch, h, Jh, F, ttype, s));
  WC_TRY(soft_adjoint(ce, ch, nullptr, acc + kAccGrad, h, Jh, ttype, lam, minl, maxh, s));
  WC_TRY(inv_adjoint(gyo, ch, h, Jh, F, ttype, s));
  WC_TRY(soft_adjoint(co, ch, nullptr, acc + kAccGrad, h, Jh, ttype, lam, minl, maxh, s));
  double hv[kAccLen];
  WC_CUDA(cudaMemcpyAsync(hv, acc, sizeof(hv), cudaMemcpyDeviceToHost, s));
  WC_TRY(take_status(s));
  *loss = hv[kAccLoss];
  for (int l = 0; l < J; l++) grad[l] = (l < Jh && l >= minl && l <= maxh) ? hv[kAccGrad + l] : 0.0;
  return WC_OK;
}

}  // namespace wc

using namespace wc;

extern "C" {

int wc_dwt_adjoint_device(const void* gin, void* gout, int64_t len, int sense, int nlevels,
                          int filter, int precision, void* stream) {
  clear_error();
  if (filter < 1 || filter > 4) return fail(WC_ERR_ARG, "unrecognised filter %d", filter);
  if (sense != 0 && sense != 1) return fail(WC_ERR_ARG, "sense must be 1 or 0");
  if (precision < 0 || precision > 2) return fail(WC_ERR_ARG, "unknown precision %d", precision);
  const int J = check_levels(len, nlevels, filter_len(filter));
  if (J == 0) return fail(WC_ERR_LEVELS, "nlevels %d invalid for length %lld", nlevels, (long long)len);
  if (!gin || !gout || gin == gout) return fail(WC_ERR_ARG, "gin and gout must be distinct");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  return dwt_adjoint(gin, gout, len, sense, J, filter, precision, s);
}

int wc_modwt_adjoint_device(double* gx, double* gxmod, int64_t len, int sense, int nlevels,
                            int filter, void* stream) {
  clear_error();
  if (filter < 1 || filter > 4) return fail(WC_ERR_ARG, "unrecognised filter %d", filter);
  if (sense != 0 && sense != 1) return fail(WC_ERR_ARG, "sense must be 1 or 0");
  const int J = check_levels(len, nlevels, filter_len(filter));
  if (J == 0) return fail(WC_ERR_LEVELS, "nlevels %d invalid for length %lld", nlevels, (long long)len);
  if (!gx || !gxmod) return fail(WC_ERR_ARG, "null pointer");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  return modwt_adjoint(gx, gxmod, len, sense, J, filter, s);
}

int wc_soft_threshold_adjoint_device(const double* coef, const double* gout, double* gcoef,
                                     double* glambda, int64_t len, int nlevels, int ttype,
                                     const double* lambda, int minlevel, int maxlevel,
                                     void* stream) {
  clear_error();
  if (!coef || !gout || !glambda || !lambda) return fail(WC_ERR_ARG, "null pointer");
  if (ttype != 0 && ttype != 1) return fail(WC_ERR_ARG, "transform type %d", ttype);
  if (nlevels < 1 || nlevels > kMaxLevels) return fail(WC_ERR_LEVELS, "nlevels %d", nlevels);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  WC_CUDA(cudaMemsetAsync(glambda, 0, sizeof(double) * (size_t)nlevels, s));
  return soft_adjoint(coef, gout, gcoef, glambda, len, nlevels, ttype, lambda, minlevel,
                      maxlevel, s);
}

}  // extern "C"

extern "C" {

int wc_loss_grad(const double* x, int64_t len, int nlevels, int filter, int ttype, int loss_type,
                 const double* lambda, int minlevel, int maxlevel, double sigma, double eps,
                 double* loss, double* grad, double* sigma_used, void* stream) {
  clear_error();
  if (filter < 1 || filter > 4) return fail(WC_ERR_ARG, "unrecognised filter %d", filter);
  if (ttype != 0 && ttype != 1) return fail(WC_ERR_ARG, "transform type %d", ttype);
  if (loss_type != WC_LOSS_SURE && loss_type != WC_LOSS_CV)
    return fail(WC_ERR_ARG, "unknown loss %d", loss_type);
  if (!x || !lambda || !loss || !grad) return fail(WC_ERR_ARG, "null pointer");
  const int J = check_levels(len, nlevels, filter_len(filter));
  if (J == 0) return fail(WC_ERR_LEVELS, "nlevels %d invalid for length %lld", nlevels, (long long)len);
  if (minlevel < 0 || maxlevel >= J || minlevel > maxlevel)
    return fail(WC_ERR_LEVELS, "level range [%d, %d] invalid for %d levels", minlevel, maxlevel, J);
  if (!(eps >= 0.0)) return fail(WC_ERR_ARG, "eps must be >= 0");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  if (loss_type == WC_LOSS_SURE)
    return sure_loss_grad(x, len, J, filter, ttype, lambda, minlevel, maxlevel, sigma, eps, loss,
                          grad, sigma_used, s);
  if (J < 2) return fail(WC_ERR_LEVELS, "cross-validation needs at least 2 levels");
  if (check_levels(len / 2, J - 1, filter_len(filter)) == 0)
    return fail(WC_ERR_LEVELS, "half-length signals cannot take %d levels", J - 1);
  if (sigma_used) *sigma_used = 0.0;
  return cv_loss_grad(x, len, J, filter, ttype, lambda, minlevel, maxlevel, loss, grad, s);
}

}  // extern "C"
