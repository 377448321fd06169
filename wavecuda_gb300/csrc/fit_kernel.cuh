#pragma once
// Per-level soft-threshold tuning by gradient descent, for a batch of
// equal-length signals in one persistent launch.  No counterpart in the
// reference: it replaces the single golden-section CV threshold of
// thresh.cpp:203-342 by one threshold per level, fitted to the SURE or the
// two-fold CV loss through the adjoints of the inverse transform and of soft
// thresholding (the same operators as adjoint.cu, here as block-level code).
//
// Each CTA pulls a signal from a work queue and runs, with no host round
// trip:
//   forward transform once (the coefficients do not depend on lambda);
//   sigma = MAD of the finest details (unless given);
//   per iteration: soft threshold per level fused into the inverse
//   transform -> residual (SURE) or interpolation residual (CV) and its
//   cotangent -> adjoint of the inverse (a forward transform of the
//   cotangent, recomputed level by level and never stored) reduced on the fly
//   against the coefficients into the per-level gradient (and, for SURE, the
//   smoothed kept counts of the divergence term) -> an Adam step on
//   u = lambda / sigma in thread 0;
//   final smoothing with the best thresholds seen.
// Bulk arithmetic is in the precision policy P (FP32, or double-float on
// FP64 data); per-thread partial sums are FP32 and block totals FP64.
//
// Loss definitions (as wc_loss_grad, adjoint.cu):
//   SURE = ||f - y||^2 - n sigma^2 + 2 sigma^2 div,  div = n - sum over the
//     thresholded levels of kappa_l (count_l - kept_l), kept_l smoothed by a
//     logistic step of width eps = eps_rel sigma; kappa_l = 1 (DWT) or
//     2^-(l+1) (MODWT, the diagonal of synthesis times analysis);
//   CV = interp_mse (thresh.cpp:344-385) of the even/odd halves transformed
//     with J-1 levels, half levels [minl, min(maxl, J-2)] thresholded.
// The CV thresholds are rescaled by 1/sqrt(1 - log 2 / log n) for the full
// signal (thresh.cpp:326); levels above J-2 take the level J-2 value.
#include <math.h>

#include "batch_kernel.cuh"
#include "wc_fit.h"

namespace wc {
namespace {

constexpr int FT = 256;  // threads per CTA (two CTAs per SM)

template <class V>
__device__ __forceinline__ float vhi(V v) {
  if constexpr (std::is_same<V, dd>::value) return v.hi + v.lo;
  else return (float)v;
}

template <class V>
__device__ __forceinline__ V from_f(float f) {
  if constexpr (std::is_same<V, dd>::value) return dd{f, 0.f};
  else return (V)f;
}

// FP32 view of a stored value without an FP64 instruction.
template <class T>
__device__ __forceinline__ float tf(T x) {
  if constexpr (std::is_same<T, double>::value) {
    const dd v = dd_from_double(x);
    return v.hi + v.lo;
  } else {
    return (float)x;
  }
}

template <class P>
struct FitShared {
  ThL<P> th;
  PipeShared pipe;
  double lam[kLvMax];
  double g[kLvMax], k[kLvMax], dk[kLvMax];
  double u[kLvMax], m[kLvMax], v[kLvMax], best_u[kLvMax];
  double loss, best_loss, sigma;
};

__device__ __forceinline__ void block_add(double* dst, float part) {
  double x = part;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0 && x != 0.0) atomicAdd(dst, x);
}

// Adjoint of the inverse MODWT applied to g (the forward a-trous chain of
// g; level l's detail cotangent is kappa_l = 2^-(l+1) times its level-l
// output, a factor the caller applies), reduced against the stored details
// det (J blocks of N) for levels [minl, maxl]:
// sh.g[l] += sum -sign(c) 1{|c| >= lam_l} gd,
// and with `div`, sh.k[l] += sum phi, sh.dk[l] += sum phi (1 - phi).
template <int F, class P>
__device__ void badj_modwt(const typename P::V* g, const typename P::T* det, int64_t N, int minl,
                           int maxl, float inv_eps, bool div, typename P::V* tA,
                           typename P::V* tB, FitShared<P>& sh) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  const int64_t B = blockDim.x;
  for (int l = 0; l <= maxl; l++) {
    const V* src = (l == 0) ? g : ((l & 1) ? tA : tB);
    V* dst = (l & 1) ? tB : tA;
    const int64_t skip = (int64_t)1 << l;
    const typename P::T* cl = det + (int64_t)l * N;
    const bool acc = l >= minl;
    const bool need_s = l < maxl;
    const float lam = (float)sh.lam[l];
    float pg = 0.f, pk = 0.f, pdk = 0.f;
    // Per output: the reduction terms of one detail cotangent d against its
    // stored coefficient c.
    auto reduce = [&](float c, float dv) {
      const float ac = fabsf(c);
      if (!(ac < lam)) pg += (c < 0.f) ? dv : -dv;
      if (div) {
        if (inv_eps > 0.f) {
          const float phi = 1.f / (1.f + __expf(-(ac - lam) * inv_eps));
          pk += phi;
          pdk += phi * (1.f - phi);
        } else if (!(ac < lam)) {
          pk += 1.f;
        }
      }
    };
    bool done = false;
    if constexpr (std::is_same<P, PF32>::value) {
      // FP32: the level on 16-byte tiles, four outputs per thread.
      auto emitg = [&](int64_t i, const float (&s)[4], const float (&d)[4]) {
        if (need_s) *reinterpret_cast<float4*>(dst + i) = make_float4(s[0], s[1], s[2], s[3]);
        if (acc) {
          const float4 c4 = *reinterpret_cast<const float4*>(cl + i);
          reduce(c4.x, d[0]);
          reduce(c4.y, d[1]);
          reduce(c4.z, d[2]);
          reduce(c4.w, d[3]);
        }
      };
      if ((((uintptr_t)dst | (uintptr_t)cl) & 15) == 0)
        done = bfwd_level_vec<F, P, V>(src, N, l, emitg);
    }
    if (!done) sweep_outputs<mod_unroll<V>()>(N, [&](auto uc, int64_t i0) {
      constexpr int UU = decltype(uc)::value;
      V v[UU][L];
      float cv[UU];
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const int64_t i = i0 + u * B;
#pragma unroll
        for (int k = 0; k < L; k++) v[u][k] = src[(i + (int64_t)k * skip) & (N - 1)];
        cv[u] = acc ? tf(cl[i]) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const int64_t i = i0 + u * B;
        V s, d;
        if constexpr (F == 1) {
          d = haar_dif<P>(v[u][0], v[u][1]);
          s = haar_sum<P>(v[u][0], v[u][1]);
        } else if constexpr (std::is_same<P, PDD>::value) {
          // The cotangents only reach FP32 partial sums of the gradient, so
          // in double-float mode the adjoint sweep runs in FP32 on the high
          // parts (a plain FP32 dot product per output).
          float fd = 0.f, fs = 0.f;
#pragma unroll
          for (int k = 0; k < L; k++) {
            fd = __fmaf_rn(v[u][k].hi, (float)tap_g(F, k), fd);
            fs = __fmaf_rn(v[u][k].hi, (float)tap_h(F, k), fs);
          }
          d = dd{fd, 0.f};
          s = dd{fs, 0.f};
        } else {
          typename P::Acc ad = P::acc_init(v[u][0], tap_g(F, 0));
          typename P::Acc as = P::acc_init(v[u][0], tap_h(F, 0));
#pragma unroll
          for (int k = 1; k < L; k++) {
            ad = P::acc_add(ad, v[u][k], tap_g(F, k));
            as = P::acc_add(as, v[u][k], tap_h(F, k));
          }
          d = P::acc_fin(ad);
          s = P::acc_fin(as);
        }
        if (need_s) dst[i] = s;
        if (acc) reduce(cv[u], vhi(d));
      }
    });
    if (acc) {
      block_add(&sh.g[l], pg);
      if (div) {
        block_add(&sh.k[l], pk);
        block_add(&sh.dk[l], pdk);
      }
    }
    __syncthreads();
  }
}

// Adjoint of the inverse DWT applied to g (a forward DWT of g; orthonormal,
// kappa 1), reduced against the interleaved coefficients w as above.
template <int F, class P>
__device__ void badj_dwt(const typename P::V* g, const typename P::T* w, int64_t N, int minl,
                         int maxl, float inv_eps, bool div, typename P::V* tA, typename P::V* tB,
                         FitShared<P>& sh) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  int64_t Nl = N;
  for (int l = 0; l <= maxl; l++) {
    const V* src = (l == 0) ? g : ((l & 1) ? tA : tB);
    V* dst = (l & 1) ? tB : tA;
    const int64_t Pq = Nl >> 1;
    const bool acc = l >= minl;
    const bool need_s = l < maxl;
    const float lam = (float)sh.lam[l];
    float pg = 0.f, pk = 0.f, pdk = 0.f;
    for (int64_t q = threadIdx.x; q < Pq; q += blockDim.x) {
      V s, d;
      if constexpr (F == 1) {
        s = haar_sum<P>(src[2 * q], src[2 * q + 1]);
        d = haar_dif<P>(src[2 * q], src[2 * q + 1]);
      } else {
        V v[L];
#pragma unroll
        for (int j = 0; j < L; j++) v[j] = src[(2 * q + j) & (Nl - 1)];
        typename P::Acc as = P::acc_init(v[0], tap_h(F, 0));
        typename P::Acc ad = P::acc_init(v[0], tap_g(F, 0));
#pragma unroll
        for (int j = 1; j < L; j++) {
          as = P::acc_add(as, v[j], tap_h(F, j));
          ad = P::acc_add(ad, v[j], tap_g(F, j));
        }
        s = P::acc_fin(as);
        d = P::acc_fin(ad);
      }
      if (need_s) dst[q] = s;
      if (acc) {
        const float c = tf(w[(2 * q + 1) << l]), ac = fabsf(c);
        if (!(ac < lam)) {
          const float dv = vhi(d);
          pg += (c < 0.f) ? dv : -dv;
        }
        if (div) {
          if (inv_eps > 0.f) {
            const float phi = 1.f / (1.f + __expf(-(ac - lam) * inv_eps));
            pk += phi;
            pdk += phi * (1.f - phi);
          } else if (!(ac < lam)) {
            pk += 1.f;
          }
        }
      }
    }
    if (acc) {
      block_add(&sh.g[l], pg);
      if (div) {
        block_add(&sh.k[l], pk);
        block_add(&sh.dk[l], pdk);
      }
    }
    __syncthreads();
    Nl = Pq;
  }
}

template <int F, class P>
__device__ void badj_any(int ttype, const typename P::V* g, const typename P::T* c, int64_t N,
                         int minl, int maxl, float inv_eps, bool div, typename P::V* tA,
                         typename P::V* tB, FitShared<P>& sh) {
  if (ttype == 0) badj_dwt<F, P>(g, c, N, minl, maxl, inv_eps, div, tA, tB, sh);
  else badj_modwt<F, P>(g, c, N, minl, maxl, inv_eps, div, tA, tB, sh);
}

// Sigma: MAD of the finest details of a coefficient store of length N.
template <class T>
__device__ double bsigma(int ttype, const T* c, int64_t N, int J, double* devbuf,
                         PipeShared& pipe) {
  Src<T> src = (ttype == 0) ? Src<T>{c, N, N, 1, J, 0, 0, N / 2} : Src<T>{c, N, N, 1, 0, 0, 0, N};
  double med, mad;
  bmedian_mad(src, devbuf, pipe.sel, &med, &mad);
  return mad;
}

__device__ __forceinline__ void zero_sums(double* g, double* k, double* dk) {
  for (int i = threadIdx.x; i < kLvMax; i += blockDim.x) g[i] = k[i] = dk[i] = 0.0;
}

// Interpolation residuals of the CV loss at half index j (thresh.cpp:363-383
// in FP32): a = yhat_even - x[2j], b = yhat_odd - x[2j+1].
template <class V, class T>
__device__ __forceinline__ void cv_ab(const V* ye, const V* yo, const T* x, int64_t h, int64_t j,
                                      float& a, float& b) {
  float yie, yio;
  if (j == 0) {
    yie = vhi(yo[0]);
    yio = 0.5f * (vhi(ye[0]) + vhi(ye[1]));
  } else if (j == h - 1) {
    yio = vhi(ye[h - 1]);
    yie = 0.5f * (vhi(yo[j]) + vhi(yo[j - 1]));
  } else {
    yio = 0.5f * (vhi(ye[j]) + vhi(ye[j + 1]));
    yie = 0.5f * (vhi(yo[j]) + vhi(yo[j - 1]));
  }
  a = yie - tf(x[2 * j]);
  b = yio - tf(x[2 * j + 1]);
}

template <int F, class P>
__device__ __noinline__ void fit_one(const FitArgs& a, int sig, CtaScratch cs, FitShared<P>& sh) {
  using T = typename P::T;
  using V = typename P::V;
  const int64_t n = a.n, h = n / 2;
  const int J = a.J, tt = a.ttype;
  const bool mod = tt == 1, cv = a.loss == WC_LOSS_CV;
  double* x = a.data + (int64_t)sig * n;
  FitResult* res = a.res + sig;

  T* xt = cs.take<T>(n);
  T* c = cs.take<T>(mod ? (int64_t)J * n : n);
  T* cJ = cs.take<T>(mod ? n : 1);
  V* tA = cs.take<V>(n);
  V* tB = cs.take<V>(n);
  V* fh = cs.take<V>(n);
  double* devbuf = cs.take<double>(n);
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) xt[i] = (T)x[i];
  __syncthreads();

  // Loss-specific stores.
  const int Jl = cv ? J - 1 : J;          // levels of the transforms the loss sees
  const int64_t nl = cv ? h : n;          // their length
  const int maxl = cv ? min(a.maxl, J - 2) : a.maxl;
  const int minl = a.minl;
  T *ce = nullptr, *ceJ = nullptr, *co = nullptr, *coJ = nullptr;
  V *ye = nullptr, *yo = nullptr, *gye = nullptr, *gyo = nullptr;
  if (cv) {
    ce = cs.take<T>(mod ? (int64_t)Jl * h : h);
    ceJ = cs.take<T>(mod ? h : 1);
    co = cs.take<T>(mod ? (int64_t)Jl * h : h);
    coJ = cs.take<T>(mod ? h : 1);
    ye = cs.take<V>(h);
    yo = cs.take<V>(h);
    gye = cs.take<V>(h);
    gyo = cs.take<V>(h);
    // halves in xt's storage order: even half into c, odd half into c + h
    T* ev = c;
    T* od = c + h;
    for (int64_t j = threadIdx.x; j < h; j += blockDim.x) {
      ev[j] = xt[2 * j];
      od[j] = xt[2 * j + 1];
    }
    __syncthreads();
    fwd_any<F, P, T>(tt, ev, ce, ceJ, h, Jl, tA, tB);
    fwd_any<F, P, T>(tt, od, co, coJ, h, Jl, tA, tB);
  } else {
    fwd_any<F, P, T>(tt, xt, c, cJ, n, J, tA, tB);
  }

  double sigma = a.sigma;
  if (!(sigma > 0.0)) sigma = bsigma<T>(tt, cv ? ce : c, nl, Jl, devbuf, sh.pipe);
  const float inv_eps = (a.eps_rel > 0.0 && sigma > 0.0) ? (float)(1.0 / (a.eps_rel * sigma)) : 0.f;

  if (threadIdx.x == 0) {
    sh.sigma = sigma;
    sh.best_loss = 1e300;
    for (int l = 0; l < kLvMax; l++) {
      const double lam0 = (l < J) ? (a.has_lam0 ? a.lam0[l] : a.sq2logn * sigma) : 0.0;
      sh.u[l] = sigma > 0.0 ? lam0 / sigma : 0.0;
      sh.lam[l] = lam0;
      sh.best_u[l] = sh.u[l];
      sh.m[l] = sh.v[l] = 0.0;
      sh.th.t[l] = to_v<P>(lam0);
    }
    sh.th.minl = minl;
    sh.th.maxl = maxl;
  }
  __syncthreads();

  const double s2 = sigma * sigma;
  const bool valid = minl <= maxl && maxl < Jl && sigma > 0.0;
  const int iters = valid ? a.iters : 0;
  if (!valid && threadIdx.x == 0) {
    res->loss0 = 0.0;
    for (int l = 0; l < kLvMax; l++) res->grad0[l] = 0.0;
  }
  for (int it = 0; valid && it <= iters; it++) {
    // ---- loss and gradient at sh.lam
    if (threadIdx.x == 0) sh.loss = 0.0;
    zero_sums(sh.g, sh.k, sh.dk);
    __syncthreads();
    if (!cv) {
      inv_any<F, P, V>(tt, c, cJ, (const V*)nullptr, fh, n, J, sh.th, tA, tB);
      float pl = 0.f;
      int64_t i0 = threadIdx.x;
      if constexpr (std::is_same<P, PF32>::value) {
        // four residuals per thread and step (scratch slices are 256-byte
        // aligned); the last n % 4 one at a time below
        float4* f4 = reinterpret_cast<float4*>(fh);
        const float4* x4 = reinterpret_cast<const float4*>(xt);
        for (int64_t i = threadIdx.x; i < n / 4; i += blockDim.x) {
          const float4 a = f4[i], b = x4[i];
          const float r0 = a.x - b.x, r1 = a.y - b.y, r2 = a.z - b.z, r3 = a.w - b.w;
          pl += r0 * r0;
          pl += r1 * r1;
          pl += r2 * r2;
          pl += r3 * r3;
          f4[i] = make_float4(2.f * r0, 2.f * r1, 2.f * r2, 2.f * r3);
        }
        i0 = (n / 4) * 4 + threadIdx.x;
      }
      for (int64_t i = i0; i < n; i += blockDim.x) {
        float r;
        if constexpr (std::is_same<V, dd>::value) {
          const dd e = P::sub(fh[i], P::ld(xt[i]));
          r = e.hi + e.lo;
        } else {
          r = vhi(fh[i]) - tf(xt[i]);
        }
        pl += r * r;
        fh[i] = from_f<V>(2.f * r);
      }
      block_add(&sh.loss, pl);
      __syncthreads();
      badj_any<F, P>(tt, fh, c, n, minl, maxl, inv_eps, true, tA, tB, sh);
    } else {
      inv_any<F, P, V>(tt, ce, ceJ, (const V*)nullptr, ye, h, Jl, sh.th, tA, tB);
      inv_any<F, P, V>(tt, co, coJ, (const V*)nullptr, yo, h, Jl, sh.th, tA, tB);
      float pl = 0.f;
      for (int64_t k = threadIdx.x; k < h; k += blockDim.x) {
        float ak, bk;
        cv_ab(ye, yo, xt, h, k, ak, bk);
        pl += ak * ak + bk * bk;
        float go = (k == 0) ? ak : 0.5f * ak;
        float ge = (k == h - 1) ? bk : 0.5f * bk;
        if (k + 1 <= h - 1) {
          float a1, b1;
          cv_ab(ye, yo, xt, h, k + 1, a1, b1);
          go += 0.5f * a1;
        }
        if (k >= 1 && k - 1 <= h - 2) {
          float a0, b0;
          cv_ab(ye, yo, xt, h, k - 1, a0, b0);
          ge += 0.5f * b0;
        }
        gyo[k] = from_f<V>(go);
        gye[k] = from_f<V>(ge);
      }
      block_add(&sh.loss, 0.5f * pl);
      __syncthreads();
      badj_any<F, P>(tt, gye, ce, h, minl, maxl, 0.f, false, tA, tB, sh);
      badj_any<F, P>(tt, gyo, co, h, minl, maxl, 0.f, false, tA, tB, sh);
    }
    // ---- loss, gradient and the Adam step (thread 0)
    if (threadIdx.x == 0) {
      double loss = sh.loss, grad[kLvMax];
      if (!cv) {
        double dv = (double)n;
        for (int l = minl; l <= maxl; l++) {
          const double kap = mod ? ldexp(1.0, -(l + 1)) : 1.0;
          const double cnt = mod ? (double)n : (double)(n >> (l + 1));
          dv -= kap * (cnt - sh.k[l]);
        }
        loss = loss - (double)n * s2 + 2.0 * s2 * dv;
      }
      for (int l = 0; l < kLvMax; l++) {
        double gl = 0.0;
        if (l >= minl && l <= maxl) {
          const double kap = mod ? ldexp(1.0, -(l + 1)) : 1.0;
          gl = kap * sh.g[l];
          if (!cv && inv_eps > 0.f) gl += 2.0 * s2 * kap * (-sh.dk[l] * (double)inv_eps);
        }
        grad[l] = gl;
      }
      if (it == 0) {
        res->loss0 = loss;
        for (int l = 0; l < kLvMax; l++) res->grad0[l] = grad[l];
      }
      if (loss < sh.best_loss) {
        sh.best_loss = loss;
        for (int l = 0; l < kLvMax; l++) sh.best_u[l] = sh.u[l];
      }
      const double b1 = 0.9, b2 = 0.999;
      const double c1 = 1.0 - pow(b1, (double)(it + 1)), c2 = 1.0 - pow(b2, (double)(it + 1));
      for (int l = minl; l <= maxl; l++) {
        const double gu = grad[l] * sigma;
        sh.m[l] = b1 * sh.m[l] + (1.0 - b1) * gu;
        sh.v[l] = b2 * sh.v[l] + (1.0 - b2) * gu * gu;
        const double den = sqrt(sh.v[l] / c2);
        if (den > 0.0) sh.u[l] = fmax(0.0, sh.u[l] - a.lr * (sh.m[l] / c1) / den);
        sh.lam[l] = sh.u[l] * sigma;
        sh.th.t[l] = to_v<P>(sh.lam[l]);
      }
    }
    __syncthreads();
  }

  // ---- final thresholds for the full signal and the smoothing
  if (threadIdx.x == 0) {
    const double sc = cv ? 1.0 / a.rescale : 1.0;
    for (int l = 0; l < kLvMax; l++) {
      double lf = 0.0;
      if (valid && l >= a.minl && l <= a.maxl) lf = sh.best_u[min(l, maxl)] * sigma * sc;
      sh.lam[l] = lf;
      sh.th.t[l] = to_v<P>(lf);
      res->lambda[l] = lf;
    }
    sh.th.minl = valid ? a.minl : 1 << 30;
    sh.th.maxl = valid ? a.maxl : -1;
    res->loss = valid ? sh.best_loss : 0.0;
    res->sigma = sigma;
    res->iterations = iters;
    res->status = valid ? 0 : 1;
  }
  __syncthreads();
  if (a.smooth && valid) {
    if (cv) fwd_any<F, P, T>(tt, xt, c, cJ, n, J, tA, tB);
    if constexpr (std::is_same<T, double>::value) {
      inv_any<F, P, double>(tt, c, cJ, (const double*)nullptr, x, n, J, sh.th, tA, tB);
    } else {
      inv_any<F, P, T>(tt, c, cJ, (const T*)nullptr, xt, n, J, sh.th, tA, tB);
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = (double)xt[i];
      __syncthreads();
    }
  }
}

template <class P>
__global__ void __launch_bounds__(FT, 2) fit_batch_kernel(FitArgs a) {
  __shared__ FitShared<P> sh;
  __shared__ int s_sig;
  CtaScratch cs{a.scratch + (size_t)blockIdx.x * a.scratch_per_cta, 0};
  while (true) {
    if (threadIdx.x == 0) s_sig = atomicAdd(a.counter, 1);
    __syncthreads();
    const int k = s_sig;
    __syncthreads();
    if (k >= a.nsig) break;
    cs.off = 0;
    switch (a.F) {
      case 1: fit_one<1, P>(a, k, cs, sh); break;
      case 2: fit_one<2, P>(a, k, cs, sh); break;
      case 3: fit_one<3, P>(a, k, cs, sh); break;
      case 4: fit_one<4, P>(a, k, cs, sh); break;
    }
    __syncthreads();
  }
}

}  // namespace

template <class P>
int fit_launch_p(const FitArgs& a, int grid, cudaStream_t s) {
  constexpr size_t smem = mod_tile_smem<typename P::V>();
  WC_CUDA(cudaFuncSetAttribute(fit_batch_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  fit_batch_kernel<P><<<grid, FT, smem, s>>>(a);
  return after_launch("fit_batch_kernel");
}

template <class P>
int fit_blocks_per_sm_p() {
  constexpr size_t smem = mod_tile_smem<typename P::V>();
  int per = 0;
  if (cudaFuncSetAttribute(fit_batch_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fit_batch_kernel<P>, FT, smem) !=
          cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return per < 1 ? 1 : per;
}

}  // namespace wc
