// Batched smoothing: descriptors shared by the persistent kernel (batch_kernel.cuh)
// and its host-side plan (batch_plan.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace wc {

struct BatchDesc {
  int64_t off, n;           // signal = data[off .. off+n)
  int J, ttype, F, threshtype, hardness, minl, maxl;
  int pair;                 // 0: one CTA; k > 0: its CV search is shared with a
                            // second CTA through pairs[k - 1]
  double thresh, tol;       // manual threshold; CV tolerance
  double sq_n, sq_nm1;      // sqrt(2 log n), sqrt(2 log(n-1)) from the host libm
  double rescale;           // sqrt(1 - log 2 / log n)
};

struct BatchResult {
  double thresh, thresh_univ, min_margin;
  int iterations, status;
  long long kept, zeroed;
};

// Meeting point of the two CTAs that share a signal's CV search (zeroed
// before every launch).  The leader runs the signal's pipeline in its own
// scratch; the partner forwards the odd half, inverts the odd half at every
// golden step and computes half of the loss terms.
struct BatchPair {
  unsigned int arrive;      // barrier arrivals of both CTAs
  unsigned int leader;      // leader's CTA index + 1, published when it starts
  unsigned int pad0[2];
  double t_univ;            // the search's upper bound, from the leader
  float part[2][2];         // double-float loss partials (hi, lo) of leader / partner
  unsigned int pad1[22];
};
static_assert(sizeof(BatchPair) == 128, "one 128-byte line per pair");

struct BatchArgs {
  const BatchDesc* desc;
  BatchResult* res;
  const int* order;         // queue units: i = signal i (its leader when paired),
                            // -(i + 1) = the partner of paired signal i
  int* counter;             // work-queue head
  int nunits;
  double* data;             // all signals, FP64, smoothed in place
  char* scratch;            // grid * scratch_per_cta bytes
  size_t scratch_per_cta;
  BatchPair* pairs;         // one per paired signal
  unsigned int* status;     // status word (bit 0: a bounded wait gave up)
  unsigned long long* trace;  // nullptr, or per queue unit: start ns, end ns, CTA
};

size_t batch_scratch_bytes(const BatchDesc& d, int prec);
int batch_launch(const BatchArgs& a, int prec, int grid, cudaStream_t s);
int batch_max_ctas(int prec);

// Per-precision instantiations of the persistent kernel (batch_exact.cu,
// batch_fast.cu, batch_f32.cu): launch, and resident CTAs per SM.
int batch_launch_exact(const BatchArgs& a, int grid, cudaStream_t s);
int batch_launch_fast(const BatchArgs& a, int grid, cudaStream_t s);
int batch_launch_f32(const BatchArgs& a, int grid, cudaStream_t s);
int batch_blocks_per_sm_exact();
int batch_blocks_per_sm_fast();
int batch_blocks_per_sm_f32();

}  // namespace wc
