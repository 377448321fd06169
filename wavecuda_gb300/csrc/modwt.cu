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
// Row view.  A level whose taps are d = 2^l0 apart splits the signal into d
// interleaved sequences: element (m, r) = x[r + m d], r < d, m < n/d, and the
// taps of (m, r) are rows m + k (forward) or m - k (inverse) of the same
// column.  The next level's taps are rows m + 2k, and so on.  A CTA stages a
// tile of C adjacent columns (C = min(d, 32): each row segment is contiguous
// in memory) by M + halo rows in shared memory, converting each value once,
// and runs several levels inside the tile; only the levels' outputs (and,
// for the inverse, the group's final scaling sequence) touch HBM.  The
// forward fuses NF levels (halo (L-1)(2^NF - 1) rows to the right); the
// inverse fuses NI levels (halo (L-1)(2^NI - 1) rows to the left), so its
// traffic is NI + 2 sequences per NI levels instead of 3 per level.  Every
// output is computed with the reference's term order, so WC_F64_EXACT stays
// bit-identical however the levels are grouped.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <vector>

#include "wc_bulk.cuh"
#include "wc_common.cuh"
#include "wc_dd.cuh"
#include "wc_taps2.cuh"
#include "wc_modwt_math.cuh"
#include "wc_modwt_vec.cuh"
#include "wc_cvfused.h"

namespace wc {
namespace {

constexpr int kThreads = 256;

// Forward levels l0 .. l0+NF-1.  Tile: columns r0 .. r0+C-1, rows m0 ..
// m0+M-1 of the row view with unit d0 = 2^l0 (nrows = n / d0 rows).
template <int F, class P, int NF>
__global__ void __launch_bounds__(kThreads)
modwt_fwd_tiled(const typename P::T* __restrict__ X, typename P::T* __restrict__ xmod,
                int64_t n, int l0, int C, int M) {
  using V = typename P::V;
  constexpr int L = filter_len(F);
  constexpr int HR = (L - 1) * ((1 << NF) - 1);       // input halo rows
  constexpr int H1 = (NF == 2) ? 2 * (L - 1) : 0;     // extra level-l0 rows kept
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* In = reinterpret_cast<V*>(smem_raw);
  V* S1 = In + (M + HR) * C;
  const int64_t d0 = (int64_t)1 << l0, nrows = n >> l0;
  const int64_t nb = d0 / C;
  const int64_t r0 = (blockIdx.x % nb) * C, m0 = (blockIdx.x / nb) * M;
  const int cs = __ffs(C) - 1;  // C is a power of two
  const int tot = (M + HR) * C;
  // Raw values arrive by per-thread asynchronous copies (all in flight at
  // once), then each thread converts its own in place.
  using T = typename P::T;
  static_assert(sizeof(T) == sizeof(V), "in-place staging");
  T* In_raw = reinterpret_cast<T*>(In);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int row = e >> cs, c = e & (C - 1);
    cp_async_elem(In_raw + e, X + (r0 + c) + ((m0 + row) & (nrows - 1)) * d0);
  }
  cp_async_wait_all();
  if constexpr (!std::is_same<T, V>::value) {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) In[e] = P::ld(In_raw[e]);
  }
  __syncthreads();
  typename P::T* S0 = xmod + (int64_t)2 * l0 * n;
  typename P::T* D0 = S0 + n;
  const int rows1 = M + H1;
  for (int e = threadIdx.x; e < rows1 * C; e += blockDim.x) {
    const int row = e >> cs, c = e & (C - 1);
    V s, d;
    fwd_taps<F, P>(In + e, C, s, d);
    if (row < M) {
      const int64_t g = (r0 + c) + (m0 + row) * d0;
      S0[g] = P::st(s);
      D0[g] = P::st(d);
    }
    if constexpr (NF == 2) S1[e] = s;
  }
  if constexpr (NF == 2) {
    __syncthreads();
    typename P::T* S2 = S0 + 2 * n;
    typename P::T* D2 = S2 + n;
    for (int e = threadIdx.x; e < M * C; e += blockDim.x) {
      const int row = e >> cs, c = e & (C - 1);
      V s, d;
      fwd_taps<F, P>(S1 + e, 2 * C, s, d);
      const int64_t g = (r0 + c) + (m0 + row) * d0;
      S2[g] = P::st(s);
      D2[g] = P::st(d);
    }
  }
}

// Inverse levels l0+NI-1 down to l0 (row unit d0 = 2^l0); one CTA per tile
// (modwt_inv_tile, wc_modwt_math.cuh).
template <int F, class P, int NI>
__global__ void __launch_bounds__(kThreads)
modwt_inv_tiled(const typename P::T* __restrict__ Stop, const typename P::T* __restrict__ xmod,
                typename P::T* __restrict__ out, int64_t n, int l0, int C, int M) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  modwt_inv_tile<F, P, NI>(blockIdx.x, Stop, xmod, out, n, l0, C, M, smem_raw, NoDMap{});
}

template <class P>
struct Geo {
  int C, M;
  size_t smem;
};

// Tile configuration per (filter, precision): the values a tile aims at
// (C * M) and the shared-memory budget per CTA, separately for the forward
// and inverse kernels.  Defaults below; wc_tune_modwt() replaces them with
// the fastest measured candidates.
struct ModCfg {
  int fwd_target, fwd_smem_kb, inv_target, inv_smem_kb;
  int inv_levels;  // levels fused per inverse launch (2 or 3; 0: the filter's default)
  int fwd_levels;  // levels fused per forward launch of the 16-byte tiles (1..3; 0: 2)
};

std::mutex g_mcfg_mu;
ModCfg g_mcfg[5][3];
bool g_mcfg_set[5][3] = {};

ModCfg default_mod_cfg(int prec) {
  const int t = (prec == WC_F32) ? 4096 : 2048;
  return ModCfg{t, 96, t, 96, 0, 0};
}

ModCfg get_mod_cfg(int F, int prec) {
  std::lock_guard<std::mutex> lk(g_mcfg_mu);
  if (!g_mcfg_set[F][prec]) {
    g_mcfg[F][prec] = default_mod_cfg(prec);
    g_mcfg_set[F][prec] = true;
  }
  return g_mcfg[F][prec];
}

void set_mod_cfg(int F, int prec, ModCfg c) {
  std::lock_guard<std::mutex> lk(g_mcfg_mu);
  g_mcfg[F][prec] = c;
  g_mcfg_set[F][prec] = true;
}

template <class P>
constexpr int prec_of() {
  return std::is_same<P, PExact>::value ? WC_F64_EXACT
         : std::is_same<P, PDD>::value  ? WC_F64_FAST
                                        : WC_F32;
}

// Tile shape for level unit d0: C = min(d0, 32) columns and the largest
// power-of-two row count M <= nrows with C*M <= target whose shared memory
// fits the budget.
template <class P>
Geo<P> tile_geo(int64_t n, int l0, int halo, int arrays, int lead_rows, int target,
                size_t budget) {
  using V = typename P::V;
  const int64_t d0 = (int64_t)1 << l0, nrows = n >> l0;
  const int C = (int)std::min<int64_t>(d0, 32);
  int M = (int)std::min<int64_t>(nrows, std::max(1, target / C));
  auto bytes = [&](int m) {
    return sizeof(V) * (size_t)C * (size_t)((m + halo) * arrays + lead_rows);
  };
  while (M > 1 && bytes(M) > budget) M >>= 1;
  return {C, M, bytes(M)};
}

constexpr int nf_max(int F) { return 2; }
// Levels fused per inverse launch: more levels mean fewer round trips of the
// intermediate scaling sequence through HBM but a deeper halo
// ((L-1)(2^NI - 1) rows); the tuner picks 2 or 3 per filter and precision.
int ni_of(int F, const ModCfg& c) { return c.inv_levels ? c.inv_levels : (F == 1 ? 3 : 2); }

// Vectorised tiles (wc_modwt_vec.cuh) where they apply; wc_set_modwt_vector(0)
// keeps every launch on the scalar tiles.
std::atomic<int> g_modwt_vec{1};

bool aligned16_host(const void* p) { return ((uintptr_t)p & 15) == 0; }

// The 16-byte forward tiles: 1..3 fused levels (wc_modwt_vec.cuh).  Returns
// WC_ERR_UNSUPPORTED when they do not apply to this launch.
template <int F, class P, int NF>
int launch_fwd_vec(const typename P::T* X, typename P::T* xmod, int64_t n, int l0, cudaStream_t s) {
  constexpr int L = filter_len(F);
  constexpr int W = mvec_w<P>();
  if (!g_modwt_vec.load() || !aligned16_host(X) || !aligned16_host(xmod) || n % W != 0)
    return WC_ERR_UNSUPPORTED;
  const ModCfg mc = get_mod_cfg(F, prec_of<P>());
  const size_t budget = (size_t)mc.fwd_smem_kb * 1024;
  const int64_t d0 = (int64_t)1 << l0, nrows = n >> l0;
  const int C = (int)std::min<int64_t>(d0, 32);
  int M = (int)std::min<int64_t>(nrows, std::max(1, mc.fwd_target / C));
  auto bytes = [&](int m) { return sizeof(typename P::T) * (size_t)mvec_fwd_values(L, NF, m, C, W); };
  while (M > W && bytes(M) > budget) M >>= 1;
  if (!mvec_ok(C, M, W)) return WC_ERR_UNSUPPORTED;
  const size_t smem = bytes(M);
  if (smem > 200 * 1024) return WC_ERR_UNSUPPORTED;
  auto kern = modwt_fwd_vec<F, P, NF>;
  WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t blocks = (d0 / C) * (nrows / M);
  {
    LaunchTimer lt("modwt_fwd_vec", s);
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(X, xmod, n, l0, C, M);
  }
  return after_launch("modwt_fwd_vec");
}

template <int F, class P, int NF>
int launch_fwd(const typename P::T* X, typename P::T* xmod, int64_t n, int l0, cudaStream_t s) {
  constexpr int L = filter_len(F);
  constexpr int HR = (L - 1) * ((1 << NF) - 1);
  // In: M + HR rows; S1 (NF == 2): M + 2(L-1) rows.
  const ModCfg mc = get_mod_cfg(F, prec_of<P>());
  const size_t budget = (size_t)mc.fwd_smem_kb * 1024;
  Geo<P> g = tile_geo<P>(n, l0, HR, 1, 0, mc.fwd_target, budget);
  if (NF == 2) {
    // recompute with both arrays
    using V = typename P::V;
    while (g.M > 1 && sizeof(V) * (size_t)g.C * (size_t)((g.M + HR) + (g.M + 2 * (L - 1))) > budget)
      g.M >>= 1;
    g.smem = sizeof(V) * (size_t)g.C * (size_t)((g.M + HR) + (g.M + 2 * (L - 1)));
  }
  auto kern = modwt_fwd_tiled<F, P, NF>;
  WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
  const int64_t blocks = (((int64_t)1 << l0) / g.C) * ((n >> l0) / g.M);
  {
    LaunchTimer lt("modwt_fwd_tiled", s);
    kern<<<(unsigned)blocks, kThreads, g.smem, s>>>(X, xmod, n, l0, g.C, g.M);
  }
  return after_launch("modwt_fwd_tiled");
}

template <int F, class P, int NI>
int launch_inv(const typename P::T* Stop, const typename P::T* xmod, typename P::T* out,
               int64_t n, int l0, cudaStream_t s) {
  constexpr int L = filter_len(F);
  constexpr int HR = (L - 1) * ((1 << NI) - 1);
  constexpr int W = mvec_w<P>();
  const ModCfg mc = get_mod_cfg(F, prec_of<P>());
  if (g_modwt_vec.load() && aligned16_host(Stop) && aligned16_host(xmod) && aligned16_host(out) &&
      n % W == 0) {
    const int C = (int)std::min<int64_t>((int64_t)1 << l0, 32);
    const int HRp = mvec_inv_halo(L, NI, C, W);
    const Geo<P> g = tile_geo<P>(n, l0, HRp, mvec_inv_arrays(NI), 0, mc.inv_target,
                                 (size_t)mc.inv_smem_kb * 1024);
    if (mvec_ok(g.C, g.M, W)) {
      auto kern = modwt_inv_vec<F, P, NI>;
      WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
      const int64_t blocks = (((int64_t)1 << l0) / g.C) * ((n >> l0) / g.M);
      {
        LaunchTimer lt("modwt_inv_vec", s);
        kern<<<(unsigned)blocks, kThreads, g.smem, s>>>(Stop, xmod, out, n, l0, g.C, g.M, HRp);
      }
      return after_launch("modwt_inv_vec");
    }
  }
  // Stop tile, NI detail tiles and NI - 1 intermediates.
  const int arrays = 2 * NI;
  Geo<P> g = tile_geo<P>(n, l0, HR, arrays, 0, mc.inv_target, (size_t)mc.inv_smem_kb * 1024);
  auto kern = modwt_inv_tiled<F, P, NI>;
  WC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
  const int64_t blocks = (((int64_t)1 << l0) / g.C) * ((n >> l0) / g.M);
  {
    LaunchTimer lt("modwt_inv_tiled", s);
    kern<<<(unsigned)blocks, kThreads, g.smem, s>>>(Stop, xmod, out, n, l0, g.C, g.M);
  }
  return after_launch("modwt_inv_tiled");
}

template <int F, class P>
int run_modwt(void* vx, void* vxmod, int64_t n, int sense, int J, cudaStream_t s) {
  using T = typename P::T;
  T* x = static_cast<T*>(vx);
  T* xmod = static_cast<T*>(vxmod);
  if (sense == 1) {
    const ModCfg mc = get_mod_cfg(F, prec_of<P>());
    const int nfv = mc.fwd_levels ? mc.fwd_levels : 2;
    for (int l = 0; l < J;) {
      const T* X = (l == 0) ? x : xmod + (int64_t)2 * (l - 1) * n;
      int nf = std::min(nfv, J - l);
      int r = nf == 3   ? launch_fwd_vec<F, P, 3>(X, xmod, n, l, s)
              : nf == 2 ? launch_fwd_vec<F, P, 2>(X, xmod, n, l, s)
                        : launch_fwd_vec<F, P, 1>(X, xmod, n, l, s);
      if (r == WC_ERR_UNSUPPORTED) {
        nf = std::min(nf_max(F), J - l);
        r = nf == 2 ? launch_fwd<F, P, 2>(X, xmod, n, l, s) : launch_fwd<F, P, 1>(X, xmod, n, l, s);
      }
      WC_TRY(r);
      l += nf;
    }
    return WC_OK;
  }
  const int nim = ni_of(F, get_mod_cfg(F, prec_of<P>()));
  T* tmp[2] = {nullptr, nullptr};
  if (J > nim) {
    tmp[0] = static_cast<T*>(workspace(kSlotModwt0, sizeof(T) * (size_t)n));
    tmp[1] = static_cast<T*>(workspace(kSlotModwt1, sizeof(T) * (size_t)n));
    if (!tmp[0] || !tmp[1]) return workspace_error();
  }
  const T* Stop = xmod + (int64_t)2 * (J - 1) * n;
  int g = 0;
  for (int hi = J - 1; hi >= 0; g++) {
    const int ni = std::min(nim, hi + 1);
    const int l0 = hi - ni + 1;
    T* out = (l0 == 0) ? x : tmp[g & 1];
    if (ni == 3) WC_TRY((launch_inv<F, P, 3>(Stop, xmod, out, n, l0, s)));
    else if (ni == 2) WC_TRY((launch_inv<F, P, 2>(Stop, xmod, out, n, l0, s)));
    else WC_TRY((launch_inv<F, P, 1>(Stop, xmod, out, n, l0, s)));
    Stop = out;
    hi = l0 - 1;
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

namespace {
template <class P>
int inv_groups_p(int64_t n, int J, int F, int target, CvModGroup* out, int* ngroups,
                 size_t* smem_max) {
  const int L = filter_len(F);
  const ModCfg mc = get_mod_cfg(F, prec_of<P>());
  const int nimax = F == 1 ? 3 : 2;
  int g = 0;
  size_t smax = 0;
  for (int hi = J - 1; hi >= 0; g++) {
    if (g >= kCvMaxGroups) return fail(WC_ERR_ARG, "too many MODWT level groups");
    const int ni = std::min(nimax, hi + 1);
    const int l0 = hi - ni + 1;
    const int HR = (L - 1) * ((1 << ni) - 1);
    const Geo<P> geo = tile_geo<P>(n, l0, HR, 2 * ni, 0, target > 0 ? target : mc.inv_target,
                                   (size_t)mc.inv_smem_kb * 1024);
    out[g] = CvModGroup{l0, ni, geo.C, geo.M, (((int64_t)1 << l0) / geo.C) * ((n >> l0) / geo.M)};
    smax = std::max(smax, geo.smem);
    hi = l0 - 1;
  }
  *ngroups = g;
  *smem_max = smax;
  return WC_OK;
}
}  // namespace

int modwt_inv_groups(int64_t n, int J, int F, int prec, int target, CvModGroup* out,
                     int* ngroups, size_t* smem_max) {
  switch (prec) {
    case WC_F64_EXACT: return inv_groups_p<PExact>(n, J, F, target, out, ngroups, smem_max);
    case WC_F64_FAST: return inv_groups_p<PDD>(n, J, F, target, out, ngroups, smem_max);
    case WC_F32: return inv_groups_p<PF32>(n, J, F, target, out, ngroups, smem_max);
  }
  return fail(WC_ERR_ARG, "unknown precision %d", prec);
}

}  // namespace wc

// ---------------------------------------------------------------- tiling --

namespace wc {
namespace {

int check_mod_cfg(int F, int prec, const ModCfg& c) {
  if (F < 1 || F > 4 || prec < 0 || prec > 2) return fail(WC_ERR_ARG, "bad filter/precision");
  auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  if (!pow2(c.fwd_target) || !pow2(c.inv_target) || c.fwd_target < 256 || c.inv_target < 256 ||
      c.fwd_target > 16384 || c.inv_target > 16384)
    return fail(WC_ERR_ARG, "tile targets must be powers of two in [256, 16384]");
  if (c.fwd_smem_kb < 16 || c.inv_smem_kb < 16 || c.fwd_smem_kb > 200 || c.inv_smem_kb > 200)
    return fail(WC_ERR_ARG, "shared-memory budgets must lie in [16, 200] KB");
  return WC_OK;
}

}  // namespace
}  // namespace wc

extern "C" int wc_set_modwt_tiling(int filter, int precision, int fwd_target, int fwd_smem_kb,
                                   int inv_target, int inv_smem_kb) {
  using namespace wc;
  clear_error();
  ModCfg c{fwd_target, fwd_smem_kb, inv_target, inv_smem_kb, 0, 0};
  WC_TRY(check_mod_cfg(filter, precision, c));
  c.inv_levels = get_mod_cfg(filter, precision).inv_levels;
  c.fwd_levels = get_mod_cfg(filter, precision).fwd_levels;
  set_mod_cfg(filter, precision, c);
  return WC_OK;
}

extern "C" int wc_set_modwt_inv_levels(int filter, int precision, int levels) {
  using namespace wc;
  clear_error();
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2)
    return fail(WC_ERR_ARG, "bad filter/precision");
  if (levels != 0 && levels != 2 && levels != 3)
    return fail(WC_ERR_ARG, "inverse levels per launch must be 2, 3 or 0 (default)");
  ModCfg c = get_mod_cfg(filter, precision);
  c.inv_levels = levels;
  set_mod_cfg(filter, precision, c);
  return WC_OK;
}

extern "C" int wc_set_modwt_fwd_levels(int filter, int precision, int levels) {
  using namespace wc;
  clear_error();
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2)
    return fail(WC_ERR_ARG, "bad filter/precision");
  if (levels < 0 || levels > 3)
    return fail(WC_ERR_ARG, "forward levels per launch must be 1, 2, 3 or 0 (default)");
  ModCfg c = get_mod_cfg(filter, precision);
  c.fwd_levels = levels;
  set_mod_cfg(filter, precision, c);
  return WC_OK;
}

extern "C" int wc_get_modwt_fwd_levels(int filter, int precision, int* levels) {
  using namespace wc;
  clear_error();
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2 || !levels)
    return fail(WC_ERR_ARG, "bad filter/precision/output");
  const int v = get_mod_cfg(filter, precision).fwd_levels;
  *levels = v ? v : 2;
  return WC_OK;
}

extern "C" int wc_set_modwt_vector(int enable) {
  wc::clear_error();
  wc::g_modwt_vec.store(enable ? 1 : 0);
  return WC_OK;
}

extern "C" int wc_get_modwt_inv_levels(int filter, int precision, int* levels) {
  using namespace wc;
  clear_error();
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2 || !levels)
    return fail(WC_ERR_ARG, "bad filter/precision/output");
  *levels = ni_of(filter, get_mod_cfg(filter, precision));
  return WC_OK;
}

extern "C" int wc_get_modwt_tiling(int filter, int precision, int* fwd_target, int* fwd_smem_kb,
                                   int* inv_target, int* inv_smem_kb) {
  using namespace wc;
  clear_error();
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2)
    return fail(WC_ERR_ARG, "bad filter/precision");
  const ModCfg c = get_mod_cfg(filter, precision);
  if (fwd_target) *fwd_target = c.fwd_target;
  if (fwd_smem_kb) *fwd_smem_kb = c.fwd_smem_kb;
  if (inv_target) *inv_target = c.inv_target;
  if (inv_smem_kb) *inv_smem_kb = c.inv_smem_kb;
  return WC_OK;
}

// Times the forward and the inverse MODWT (nlevels levels) of a 2^log2n
// signal for each candidate tile target and shared-memory budget (and, for
// the inverse, 2 or 3 levels per launch), and keeps the fastest of each
// direction.
extern "C" int wc_tune_modwt(int filter, int precision, int log2n, int nlevels, float* fwd_ms,
                             float* inv_ms) {
  using namespace wc;
  clear_error();
  WC_TRY(ensure_device());
  if (filter < 1 || filter > 4 || precision < 0 || precision > 2)
    return fail(WC_ERR_ARG, "bad filter/precision");
  if (log2n < 14 || log2n > 26) return fail(WC_ERR_ARG, "log2n must lie in [14, 26]");
  const int64_t n = (int64_t)1 << log2n;
  const int J = check_levels(n, nlevels, filter_len(filter));
  if (J == 0) return fail(WC_ERR_LEVELS, "nlevels %d invalid", nlevels);
  const size_t es = (precision == WC_F32) ? 4 : 8;
  void* x = nullptr;
  void* xm = nullptr;
  WC_CUDA(cudaMalloc(&x, es * (size_t)n));
  if (cudaMalloc(&xm, es * (size_t)n * 2 * (size_t)J) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(x);
    return fail(WC_ERR_NOMEM, "tuning buffers");
  }
  cudaStream_t s = lib_stream();
  if (fill_noise(x, n, es, s) != WC_OK) {
    cudaFree(x);
    cudaFree(xm);
    return fail(WC_ERR_CUDA, "tuning signal");
  }
  const ModCfg keep = get_mod_cfg(filter, precision);
  const int base = (precision == WC_F32) ? 2048 : 1024;
  std::vector<std::pair<int, int>> cand;
  for (int t : {base, 2 * base, 4 * base})
    for (int kb : {48, 72, 96}) cand.push_back({t, kb});
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float bf = 1e30f, bi = 1e30f;
  ModCfg best = keep;
  int rc = WC_OK;
  // Best of reps 2..3 of one direction under configuration c.
  auto time_dir = [&](const ModCfg& c, int sense, float* ms) {
    set_mod_cfg(filter, precision, c);
    float m = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, s);
      const int r = modwt(x, xm, n, sense, J, filter, precision, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      if (r != WC_OK) return r;
      float a = 0.f;
      cudaEventElapsedTime(&a, e0, e1);
      if (rep > 0) m = std::min(m, a);
    }
    *ms = m;
    return WC_OK;
  };
  // The forward first (the inverse reads its output), per tiling and levels
  // per launch; then the inverse.
  for (const auto& c : cand) {
    for (int nf : {1, 2, 3}) {
      float m = 0.f;
      rc = time_dir(ModCfg{c.first, c.second, keep.inv_target, keep.inv_smem_kb, keep.inv_levels, nf},
                    1, &m);
      if (rc != WC_OK) break;
      if (m < bf) {
        bf = m;
        best.fwd_target = c.first;
        best.fwd_smem_kb = c.second;
        best.fwd_levels = nf;
      }
    }
    if (rc != WC_OK) break;
  }
  for (const auto& c : cand) {
    if (rc != WC_OK) break;
    for (int ni : {2, 3}) {
      float m = 0.f;
      rc = time_dir(ModCfg{best.fwd_target, best.fwd_smem_kb, c.first, c.second, ni,
                           best.fwd_levels}, 0, &m);
      if (rc != WC_OK) break;
      if (m < bi) {
        bi = m;
        best.inv_target = c.first;
        best.inv_smem_kb = c.second;
        best.inv_levels = ni;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(xm);
  set_mod_cfg(filter, precision, rc == WC_OK ? best : keep);
  if (fwd_ms) *fwd_ms = bf;
  if (inv_ms) *inv_ms = bi;
  return rc;
}

// ---------------------------------------------------------------------------
// Packet-ordered MODWT (code 2; fHaarMODWT/bHaarMODWT, haar.cpp:305-398, and
// fDaub4MODWTpo/bDaub4MODWTpo, daub4.cpp:392-484 of the reference; C6 and
// LA8 by the same rules).  Its forward coefficients are the time-ordered
// ones stored per packet: level l's packet sh holds the (s, d) pairs of time
// positions rev(sh, l+1) + 2^(l+1) k, interleaved (convert_modwt_level,
// wavutils.cpp:569-600).  Its inverse differs in arithmetic: every packet is
// inverted one DWT level and each packet pair's two reconstructions are
// averaged (writeavpackets, wavutils.cpp:304-330).  Here the inverse works on
// the time-ordered copy: output u = st + 2^l i of level l-1 averages packet
// residue st at packet position i with residue st + 2^l at position i - 1.

namespace wc {
namespace {

template <class T>
__global__ void modwt_layout_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                                    int log2n, int J, int to_po) {
  const int64_t total = 2 * n * (int64_t)J;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += stride) {
    const int l = (int)(idx / (2 * n));
    const int64_t base = (int64_t)l * 2 * n, e = idx - base;
    const int64_t skip = (int64_t)1 << l, lenos = n >> l;
    const int64_t sh = e >> (log2n - l), w = e & (lenos - 1), k = w >> 1;
    const int64_t st = (int64_t)(__brev((unsigned)sh) >> (31 - l));
    const int64_t te = ((w & 1) ? n : 0) + st + 2 * skip * k;
    if (to_po) out[base + e] = in[base + te];
    else out[base + te] = in[base + e];
  }
}

// One value of the one-level inverse DWT of the packet whose pairs are
// (S, D)[r + 2 skip q], q < Pq, at packet position i (the arithmetic of
// bHaar / bDaub4 / bC6 / bLA8: taps in descending j, s before d).
template <int F, class P>
__device__ __forceinline__ typename P::V po_packet_inv(const typename P::T* S,
                                                       const typename P::T* D, int64_t r,
                                                       int64_t skip, int64_t Pq, int64_t i) {
  using V = typename P::V;
  const int64_t q = i >> 1;
  const bool odd = (i & 1) != 0;
  if constexpr (F == 1) {
    const V a = P::ld(S[r + 2 * skip * q]), b = P::ld(D[r + 2 * skip * q]);
    return odd ? haar_dif<P>(a, b) : haar_sum<P>(a, b);
  } else {
    constexpr int HH = filter_len(F) / 2;
    V sv[HH], dv[HH];
#pragma unroll
    for (int j = 0; j < HH; j++) {
      const int64_t p = (q - j) & (Pq - 1);
      sv[j] = P::ld(S[r + 2 * skip * p]);
      dv[j] = P::ld(D[r + 2 * skip * p]);
    }
    typename P::Acc ae = P::acc_init(sv[HH - 1], tap_h(F, 2 * (HH - 1)));
    typename P::Acc ao = P::acc_init(sv[HH - 1], tap_h(F, 2 * (HH - 1) + 1));
    ae = P::acc_add(ae, dv[HH - 1], tap_g(F, 2 * (HH - 1)));
    ao = P::acc_add(ao, dv[HH - 1], tap_g(F, 2 * (HH - 1) + 1));
#pragma unroll
    for (int j = HH - 2; j >= 0; j--) {
      ae = P::acc_add(ae, sv[j], tap_h(F, 2 * j));
      ao = P::acc_add(ao, sv[j], tap_h(F, 2 * j + 1));
      ae = P::acc_add(ae, dv[j], tap_g(F, 2 * j));
      ao = P::acc_add(ao, dv[j], tap_g(F, 2 * j + 1));
    }
    return odd ? P::acc_fin(ao) : P::acc_fin(ae);
  }
}

template <int F, class P>
__global__ void __launch_bounds__(kThreads)
modwt_po_inv_level(const typename P::T* __restrict__ S, const typename P::T* __restrict__ D,
                   typename P::T* __restrict__ out, int64_t n, int l) {
  const int64_t skip = (int64_t)1 << l, lenos = n >> l, Pq = lenos >> 1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += stride) {
    const int64_t st = u & (skip - 1), i = u >> l;
    const typename P::V a = po_packet_inv<F, P>(S, D, st, skip, Pq, i);
    const typename P::V b =
        po_packet_inv<F, P>(S, D, st + skip, skip, Pq, (i + lenos - 1) & (lenos - 1));
    out[u] = P::st(P::half(P::add(a, b)));
  }
}

unsigned po_grid(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16));
}

template <int F, class P>
int run_po_inverse(const typename P::T* xmod, typename P::T* x, int64_t n, int J,
                   cudaStream_t s) {
  using T = typename P::T;
  T* tmp[2] = {nullptr, nullptr};
  if (J > 1) {
    tmp[0] = static_cast<T*>(workspace(kSlotModwt0, sizeof(T) * (size_t)n));
    tmp[1] = static_cast<T*>(workspace(kSlotModwt1, sizeof(T) * (size_t)n));
    if (!tmp[0] || !tmp[1]) return workspace_error();
  }
  const T* S = xmod + (int64_t)2 * (J - 1) * n;
  for (int l = J - 1; l >= 0; l--) {
    T* out = (l == 0) ? x : tmp[l & 1];
    {
      LaunchTimer lt("modwt_po_inv_level", s);
      modwt_po_inv_level<F, P><<<po_grid(n), kThreads, 0, s>>>(S, xmod + (int64_t)(2 * l + 1) * n,
                                                              out, n, l);
    }
    WC_TRY(after_launch("modwt_po_inv_level"));
    S = out;
  }
  return WC_OK;
}

template <class P>
int dispatch_po_inverse(const void* xmod, void* x, int64_t n, int J, int F, cudaStream_t s) {
  using T = typename P::T;
  const T* xm = static_cast<const T*>(xmod);
  T* xo = static_cast<T*>(x);
  switch (F) {
    case 1: return run_po_inverse<1, P>(xm, xo, n, J, s);
    case 2: return run_po_inverse<2, P>(xm, xo, n, J, s);
    case 3: return run_po_inverse<3, P>(xm, xo, n, J, s);
    case 4: return run_po_inverse<4, P>(xm, xo, n, J, s);
  }
  return fail(WC_ERR_ARG, "unknown filter %d", F);
}

}  // namespace

int modwt_layout(const void* in, void* out, int64_t n, int J, int to_po, int prec,
                 cudaStream_t s) {
  int log2n = 0;
  while (((int64_t)1 << log2n) < n) log2n++;
  const int64_t total = 2 * n * (int64_t)J;
  LaunchTimer lt("modwt_layout", s);
  if (prec == WC_F32)
    modwt_layout_kernel<float><<<po_grid(total), kThreads, 0, s>>>(
        static_cast<const float*>(in), static_cast<float*>(out), n, log2n, J, to_po);
  else
    modwt_layout_kernel<double><<<po_grid(total), kThreads, 0, s>>>(
        static_cast<const double*>(in), static_cast<double*>(out), n, log2n, J, to_po);
  return after_launch("modwt_layout_kernel");
}

int modwt_po_inverse_to(void* x, const void* xmod, int64_t n, int J, int F, int prec,
                        cudaStream_t s) {
  switch (prec) {
    case WC_F64_EXACT: return dispatch_po_inverse<PExact>(xmod, x, n, J, F, s);
    case WC_F64_FAST: return dispatch_po_inverse<PDD>(xmod, x, n, J, F, s);
    case WC_F32: return dispatch_po_inverse<PF32>(xmod, x, n, J, F, s);
  }
  return fail(WC_ERR_ARG, "unknown precision %d", prec);
}

int modwt_po(void* x, void* xmod, int64_t n, int sense, int J, int F, int prec, cudaStream_t s) {
  const size_t es = (prec == WC_F32) ? 4 : 8;
  void* to = workspace(kSlotPacket, es * 2 * (size_t)n * (size_t)J);
  if (!to) return workspace_error();
  if (sense == 1) {
    WC_TRY(modwt(x, to, n, 1, J, F, prec, s));
    return modwt_layout(to, xmod, n, J, 1, prec, s);
  }
  WC_TRY(modwt_layout(xmod, to, n, J, 0, prec, s));
  return modwt_po_inverse_to(x, to, n, J, F, prec, s);
}

}  // namespace wc
