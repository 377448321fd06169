// Fused cross-validation search: the arguments shared by the persistent
// cooperative kernel (cv_fused_kernel.cuh) and its host driver (smooth.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace wc {

// Golden-section state: t0..t3 in (host-computed start), t1, t2, m1, m2,
// iterations and the smallest relative loss margin out.
struct CvFusedState {
  double t0, t1, t2, t3;
  double m1, m2, min_margin;
  double m_new;  // loss of the latest candidate (exchanged between CTAs)
  int iters, pad;
};

// One group of MODWT inverse levels l0 .. l0+ni-1 run as row-view tiles of
// C columns x M rows (ntiles tiles per half).
struct CvModGroup {
  int l0, ni, C, M;
  int64_t ntiles;
};

constexpr int kCvMaxGroups = 24;
constexpr int kCvCoarseMax = 4096;  // DWT levels with at most this many outputs run in one CTA

struct CvFusedArgs {
  const void* wcoef[2];  // coefficients of the even / odd halves (T): DWT lenh values
                         // (interleaved), MODWT 2 lenh J1 values
  const double* x;       // the noisy signal, 2 lenh FP64 values
  void* rec[4];          // reconstructions (T, lenh each): pair 0 = rec[0..1], pair 1 = rec[2..3]
  void* top[4];          // DWT: previous reconstruction's coarse slots k 2^J1 (T, lenh >> J1)
  void* tmp[2][2];       // intermediate scaling sequences per half (T, lenh each)
  double* terms;         // lenh loss terms
  double* chunk_s;       // per chunk of kSeqChunk terms: FP64 sum (any order); two
                         // buffers of chunks (the non-exact losses alternate them)
  int* chunk_e;          // binade estimate of the running sum at the chunk's start
  long long* chunk_q;    // 3 per chunk: increments for the binades chunk_e - 1 .. + 1
  long long* sub_q;      // 16 x 3 per chunk: the same for its 64-term sub-chunks
  CvFusedState* st;
  unsigned int* bar;     // grid barrier words (grid_bar_words, zero)
  unsigned int* status;  // status word (bit 0: a bounded wait gave up)
  int64_t lenh;
  int J1;                // levels of the half-length transforms
  int minl, maxl1;       // thresholded half levels (0-based)
  int hardness;
  int thr_on;            // 0: the half level range is invalid, nothing is thresholded
  double tol;
  int ngroups;           // MODWT inverse groups, coarsest first
  CvModGroup grp[kCvMaxGroups];
  int dwt_lc;            // DWT: levels J1-1 .. dwt_lc run in one CTA per half (dwt_lc > J1-1: none)
  // Optional phase timer (nullptr: off): CTA 0 adds the wall time (ns) of
  // each phase over the whole search, slots 0 .. kCvMaxGroups-1 for the
  // transform's level groups (DWT: 0 = the coarse CTA phase, 1 + k = fine
  // level k), then the loss terms, the increments and the replay.
  unsigned long long* trace;
};
constexpr int kCvTraceTerms = kCvMaxGroups, kCvTraceQ = kCvMaxGroups + 1,
              kCvTraceReplay = kCvMaxGroups + 2, kCvTraceSlots = kCvMaxGroups + 3;

// Level groups of the time-ordered MODWT inverse of an n-sample signal with
// J levels, coarsest first, as the tiled inverse runs them (tile target
// `target` values, 0 = the tuned setting), with the largest shared-memory
// size of their tiles (modwt.cu).
int modwt_inv_groups(int64_t n, int J, int F, int prec, int target, CvModGroup* out,
                     int* ngroups, size_t* smem_max);

// Per-precision instantiations (cv_fused_exact.cu, cv_fused_fast.cu,
// cv_fused_f32.cu): cooperative launch of the search for filter F and
// transform ttype (0 DWT, 1 MODWT) on `grid` CTAs with `smem` bytes of
// dynamic shared memory.
int cv_fused_launch_exact(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                          cudaStream_t s);
int cv_fused_launch_fast(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                         cudaStream_t s);
int cv_fused_launch_f32(const CvFusedArgs& a, int F, int ttype, int grid, size_t smem,
                        cudaStream_t s);
// Resident CTAs per SM of the instantiation at `smem` bytes of dynamic
// shared memory (0 when it cannot run).
int cv_fused_occupancy_exact(int F, int ttype, size_t smem);
int cv_fused_occupancy_fast(int F, int ttype, size_t smem);
int cv_fused_occupancy_f32(int F, int ttype, size_t smem);

}  // namespace wc
