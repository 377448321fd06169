// Time-ordered MODWT (haar.cpp:561-685, daub4.cpp:495-589), forward and
// inverse, for Haar, D4, C6 and LA8.  The reference has this transform only
// for Haar and D4 on the CPU (transform.cpp:53-72) and for Haar on the GPU
// (transformcuda.cu:43-76); C6 and LA8 use the same a-trous form with their
// taps:  S_l[i] = sum_k h_k S_{l-1}[i + k 2^(l-1)],  D_l[i] = sum_k g_k (...),
// inverse  X[i] = 0.5 * sum_k (h_k S[i - k s] + g_k D[i - k s]) with the even
// taps first (daub4.cpp:578-582 term order).
//
// Layout: xmod = [s_1 | d_1 | ... | s_J | d_J], each block len values.  The
// inverse reads s_J and d_1..d_J only and keeps its intermediate scaling
// sequences in workspace, so xmod is not modified.
//
// Each level is one streaming launch: thread i produces S[i], D[i] (or X[i])
// from L taps spaced 2^l apart.  Loads of neighbouring threads are
// contiguous, so every tap read is coalesced and the L-fold reuse of a value
// is served from L1/L2.
#include <algorithm>

#include "wc_common.cuh"
#include "wc_dd.cuh"

namespace wc {
namespace {

constexpr int kThreads = 256;

template <int F, class P>
__global__ void __launch_bounds__(kThreads)
modwt_fwd_level(const typename P::T* __restrict__ X, typename P::T* __restrict__ S,
                typename P::T* __restrict__ D, int64_t n, int64_t skip) {
  using V = typename P::V;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if constexpr (F == 1) {
      V a = P::ld(X[i]), b = P::ld(X[wrap(i + skip, n)]);
      D[i] = P::st(haar_dif<P>(a, b));
      S[i] = P::st(haar_sum<P>(a, b));
    } else {
      constexpr int L = filter_len(F);
      V v = P::ld(X[i]);
      typename P::Acc d = P::acc_init(v, tap_g(F, 0)), s = P::acc_init(v, tap_h(F, 0));
#pragma unroll
      for (int k = 1; k < L; k++) {
        v = P::ld(X[wrap(i + (int64_t)k * skip, n)]);
        d = P::acc_add(d, v, tap_g(F, k));
        s = P::acc_add(s, v, tap_h(F, k));
      }
      D[i] = P::st(P::acc_fin(d));
      S[i] = P::st(P::acc_fin(s));
    }
  }
}

template <int F, class P>
__global__ void __launch_bounds__(kThreads)
modwt_inv_level(typename P::T* __restrict__ Xout, const typename P::T* __restrict__ S,
                const typename P::T* __restrict__ D, int64_t n, int64_t skip) {
  using V = typename P::V;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if constexpr (F == 1) {
      const int64_t j = wrap(i - skip, n);
      V acc = P::add(P::ld(S[i]), P::ld(D[i]));
      acc = P::add(acc, P::ld(S[j]));
      acc = P::sub(acc, P::ld(D[j]));
      Xout[i] = P::st(P::mul(acc, kHInvR2));
    } else {
      constexpr int L = filter_len(F);
      typename P::Acc acc;
#pragma unroll
      for (int t = 0; t < L; t++) {
        // even taps L-2, ..., 0 then odd taps L-1, ..., 1
        const int k = (t < L / 2) ? (L - 2 - 2 * t) : (L - 1 - 2 * (t - L / 2));
        const int64_t j = wrap(i - (int64_t)k * skip, n);
        if (t == 0) acc = P::acc_init(P::ld(S[j]), tap_h(F, k));
        else acc = P::acc_add(acc, P::ld(S[j]), tap_h(F, k));
        acc = P::acc_add(acc, P::ld(D[j]), tap_g(F, k));
      }
      Xout[i] = P::st(P::half(P::acc_fin(acc)));
    }
  }
}

unsigned grid_for(int64_t n) {
  int64_t blocks = (n + kThreads - 1) / kThreads;
  return (unsigned)std::min<int64_t>(blocks, 152 * 16);
}

template <int F, class P>
int run_modwt(void* vx, void* vxmod, int64_t n, int sense, int J, cudaStream_t s) {
  using T = typename P::T;
  T* x = static_cast<T*>(vx);
  T* xmod = static_cast<T*>(vxmod);
  const unsigned grid = grid_for(n);
  if (sense == 1) {
    for (int l = 0; l < J; l++) {
      const T* X = (l == 0) ? x : xmod + (int64_t)2 * (l - 1) * n;
      {
        LaunchTimer lt("modwt_fwd_level", s);
        modwt_fwd_level<F, P><<<grid, kThreads, 0, s>>>(
            X, xmod + (int64_t)2 * l * n, xmod + (int64_t)(2 * l + 1) * n, n, (int64_t)1 << l);
      }
      WC_TRY(after_launch("modwt_fwd_level"));
    }
    return WC_OK;
  }
  T* tmp[2] = {nullptr, nullptr};
  if (J > 1) {
    tmp[0] = static_cast<T*>(workspace(kSlotModwt0, sizeof(T) * (size_t)n));
    tmp[1] = static_cast<T*>(workspace(kSlotModwt1, sizeof(T) * (size_t)n));
    if (!tmp[0] || !tmp[1]) return workspace_error();
  }
  const T* Sin = xmod + (int64_t)2 * (J - 1) * n;
  for (int l = J - 1; l >= 0; l--) {
    T* out = (l == 0) ? x : tmp[l & 1];
    {
      LaunchTimer lt("modwt_inv_level", s);
      modwt_inv_level<F, P><<<grid, kThreads, 0, s>>>(out, Sin, xmod + (int64_t)(2 * l + 1) * n,
                                                      n, (int64_t)1 << l);
    }
    WC_TRY(after_launch("modwt_inv_level"));
    Sin = out;
  }
  return WC_OK;
}

template <class P>
int dispatch_modwt(void* x, void* xmod, int64_t n, int sense, int J, int F, cudaStream_t s) {
  switch (F) {
    case 1: return run_modwt<1, P>(x, xmod, n, sense, J, s);
    case 2: return run_modwt<2, P>(x, xmod, n, sense, J, s);
    case 3: return run_modwt<3, P>(x, xmod, n, sense, J, s);
    case 4: return run_modwt<4, P>(x, xmod, n, sense, J, s);
  }
  return fail(WC_ERR_ARG, "unknown filter %d", F);
}

}  // namespace

int modwt(void* x, void* xmod, int64_t n, int sense, int J, int F, int prec, cudaStream_t s) {
  switch (prec) {
    case WC_F64_EXACT: return dispatch_modwt<PExact>(x, xmod, n, sense, J, F, s);
    case WC_F64_FAST: return dispatch_modwt<PDD>(x, xmod, n, sense, J, F, s);
    case WC_F32: return dispatch_modwt<PF32>(x, xmod, n, sense, J, F, s);
  }
  return fail(WC_ERR_ARG, "unknown precision %d", prec);
}

}  // namespace wc
