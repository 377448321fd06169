// Host-side internals shared by the library's translation units: error
// reporting, the per-device workspace, launch accounting and the device-path
// drivers that the C ABI (abi.cu) composes.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/wavecuda_gb300.h"

namespace wc {

// Records the error text for wc_last_error() and returns code.
int fail(int code, const char* fmt, ...);
// Clears the thread's error text.
void clear_error();
const char* last_error_text();

#define WC_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess)                                                   \
      return ::wc::fail(WC_ERR_CUDA, "%s failed: %s (%s:%d)", #call,         \
                        cudaGetErrorString(_e), __FILE__, __LINE__);         \
  } while (0)

#define WC_TRY(expr)          \
  do {                        \
    int _r = (expr);          \
    if (_r != WC_OK) return _r; \
  } while (0)

// Every kernel launch goes through this so that the library can report how
// many of its kernels ran (wc_kernel_launch_count) and check launch errors.
int after_launch(const char* what);
void count_launches(int64_t k);

// Brackets one kernel launch with CUDA events while profiling is on
// (wc_profile_start); a no-op otherwise.
class LaunchTimer {
 public:
  LaunchTimer(const char* name, cudaStream_t s);
  ~LaunchTimer();
 private:
  const char* name_;
  cudaStream_t s_;
  void* start_;
};

// Workspace slots.  Each slot is a device buffer grown on demand and kept
// until wc_release(); slots never alias one another.
enum Slot {
  kSlotStageA = 0,   // host-boundary staging (x / xmod in)
  kSlotStageB,       // host-boundary staging (out)
  kSlotCoarse0,      // DWT compact coarse coefficients (ping)
  kSlotCoarse1,      // DWT compact coarse coefficients (pong)
  kSlotModwt0,       // MODWT inverse intermediate (ping)
  kSlotModwt1,       // MODWT inverse intermediate (pong)
  kSlotSelect,       // radix-select histograms and results
  kSlotSelectData,   // radix-select materialised keys
  kSlotCv,           // cross-validation vectors
  kSlotCvTerms,      // cross-validation loss terms
  kSlotReduce,       // reductions (counts, sums)
  kSlotConvert,      // FP32 conversions at the boundary
  kSlotStatus,       // device status word
  kSlotBatch,        // batched smoothing (descriptors, results, CTA scratch)
  kSlotAdjoint,      // loss / gradient evaluation (coefficients, cotangents)
  kSlotTune,         // batched threshold tuning (coefficients, state)
  kSlotPacket,       // packet-ordered MODWT: time-ordered copy of the coefficients
  kSlotBatchScratch, // batched smoothing through the host-buffer call: CTA scratch
  kSlotHostCoarse,   // host-streamed DWT: coarse slots gathered from the host array
  kNumSlots
};

// Returns a device buffer of at least `bytes` for `slot` on the current
// device (nullptr plus an error on failure).
void* workspace(Slot slot, size_t bytes);
int workspace_error();  // WC_ERR_NOMEM / WC_ERR_CUDA of the last workspace() failure

// Per-device status word that kernels OR error bits into (bit 0: a bounded
// device-side wait gave up); zero-initialised when first created.
unsigned int* device_status_word();
// The same word if it already exists on the current device (nullptr
// otherwise); never allocates.
unsigned int* existing_status_word();
// Synchronises s, then reads and clears the status word: WC_ERR_TIMEOUT (with
// the error text set) when a bounded wait gave up, else WC_OK.  Every
// host-buffer call runs it after its device work and before it writes the
// caller's buffers.
int take_status(cudaStream_t s);
// Status word of the allocation-free DWT (inside its static device array) on
// the current device: the _if_known form returns nullptr until that entry
// point has looked the array up on this device and never calls the runtime's
// symbol lookup; noalloc_status_word looks it up.
unsigned int* noalloc_status_word_if_known();
int noalloc_status_word(unsigned int** w);

// The library's own non-blocking stream on the current device.
cudaStream_t lib_stream();

// Writes n pseudo-random values in [-1, 1) (FP64 for es == 8, FP32 for
// es == 4) on stream s: the autotuners' test signal.
int fill_noise(void* x, int64_t n, size_t es, cudaStream_t s);
// Makes sure a CUDA device is usable and current.
int ensure_device();

// ---------------------------------------------------------------- drivers --
// All drivers take device pointers and a stream, validate nothing that the
// ABI layer already validated, and return a WC_* status.

// Level count after check_len_levels (0 = invalid).
int check_levels(int64_t n, int nlevels, int filterlen);

// DWT out of place (in != out), interleaved layout.
int dwt(const void* in, void* out, int64_t n, int sense, int J, int F, int prec,
        cudaStream_t s);

// In-place DWT of a host array the GPU can address (FP64 data; exact or
// double-float arithmetic), streamed over the host link in chunks.
// Returns WC_ERR_UNSUPPORTED, with nothing enqueued, when the signal is too
// short for chunking or the precision is FP32.  Enqueues on s; the caller
// synchronises.
int dwt_host_inplace(double* x, int64_t n, int sense, int J, int F, int prec, cudaStream_t s);

// Packet-ordered MODWT (code 2, haar.cpp:305-398, daub4.cpp:392-484).
// FWD: x -> xmod in packet order.  BWD: xmod (packet order, not modified) ->
// x, averaging packet-pair reconstructions as the reference does.
int modwt_po(void* x, void* xmod, int64_t n, int sense, int J, int F, int prec, cudaStream_t s);
// Per-level permutation of a 2*n*J MODWT array between time order and
// packet order (to_po 1: time -> packet), out of place.
int modwt_layout(const void* in, void* out, int64_t n, int J, int to_po, int prec,
                 cudaStream_t s);
// Inverse of a time-ordered coefficient array with the packet-ordered
// transform's arithmetic (xmod not modified).
int modwt_po_inverse_to(void* x, const void* xmod, int64_t n, int J, int F, int prec,
                        cudaStream_t s);

// Time-ordered MODWT.  FWD: x -> xmod.  BWD: xmod -> x (xmod not modified).
int modwt(void* x, void* xmod, int64_t n, int sense, int J, int F, int prec,
          cudaStream_t s);

// In-place threshold of a DWT (x) or MODWT (xmod) in levels [minl, maxl].
int threshold(void* data, int64_t n, int J, int ttype, double t, int hardness,
              int minl, int maxl, int prec, cudaStream_t s);

// univ_thresh (thresh.cpp:170-201) of a transformed FP64 vector; synchronous.
int univ_thresh(const double* data, int64_t n, int J, int ttype, int minl,
                int maxl, cudaStream_t s, double* out);

// Exact k-th smallest (0-based) of the FP64 values described by the
// selection source; synchronous.
struct SelectSource {
  const double* base;  // first element
  int64_t seg_len;     // elements per segment
  int64_t seg_stride;  // distance between segment starts (elements)
  int64_t nseg;        // number of segments
};
int median_mad(const SelectSource& src, int64_t count, cudaStream_t s,
               double* median, double* mad);

// Kept/zeroed detail counts of a transformed FP64 vector; synchronous.
int count_kept(const double* data, int64_t n, int J, int ttype, double t,
               int minl, int maxl, cudaStream_t s, int64_t* kept,
               int64_t* zeroed);

// Full smoothing on a device-resident signal x (FP64, n values), replaced by
// the smoothed signal.  threshtype 0 manual, 1 univ, 2 cv.
int smooth(double* x, int64_t n, int J, int ttype, int F, int threshtype,
           double* thresh, int hardness, int minl, int maxl, double tol,
           int prec, cudaStream_t s, wc_smooth_info* info);

}  // namespace wc
