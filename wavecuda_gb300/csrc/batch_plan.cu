// Host side of batched smoothing: validation, per-signal constants, the
// work-queue order (largest work first, the CV searches too long for one CTA
// split over two), per-CTA scratch sizing, the grid size (autotuned on
// request), and a CUDA graph that replays the queue reset and the
// persistent launch.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <mutex>
#include <numeric>
#include <vector>

#include "wc_batch.h"
#include "wc_common.cuh"

struct wc_batch_plan_s {
  int nsig = 0;
  int npairs = 0;  // signals whose CV search two CTAs share
  int nunits = 0;  // queue units: nsig + npairs
  int prec = 0;
  int grid = 0;
  size_t scratch_per_cta = 0;
  int64_t total = 0;  // elements spanned by the batch (max off + n)
  wc::BatchDesc* d_desc = nullptr;
  wc::BatchResult* d_res = nullptr;
  int* d_order = nullptr;
  int* d_counter = nullptr;
  wc::BatchPair* d_pairs = nullptr;
  unsigned int* status = nullptr;
  unsigned long long* d_trace = nullptr;  // per-unit timing (WAVECUDA_BATCH_TRACE)
  std::vector<int> order;                 // host copy of the queue, for the trace
  std::vector<wc::BatchDesc> desc;
  char* d_scratch = nullptr;
  bool own_scratch = true;  // false: the scratch is the library workspace
  size_t scratch_bytes = 0;
  // graph cache
  cudaGraphExec_t exec = nullptr;
  double* graph_data = nullptr;
  cudaStream_t graph_stream = nullptr;
  int graph_grid = 0;
};

namespace wc {
namespace {

// Work estimates (in multiply-adds) of a signal's pipeline: the forward
// transform and final inverse, the universal threshold's selections and, for
// CV, the forward of both halves and about 40 golden steps, each an inverse
// of both halves plus the loss terms and their serial sum.  `solo`: one CTA
// does everything; `leader` / `partner`: the busy time of the two CTAs of a
// pair, which split the half-signal work and the terms but both replay the
// serial sum, and whose partner idles through the leader's first stage.
struct Cost {
  double solo, leader, partner;
};
Cost cost_of(const BatchDesc& d) {
  const double L = (double)filter_len(d.F), n = (double)d.n;
  const bool mod = d.ttype == 1;
  const double fwd = mod ? n * d.J * 2.0 * L : n * 2.0 * L;  // one transform
  const double sel = d.threshtype >= 1 ? n * (mod ? d.J : 1) * 4.0 : 0.0;
  if (d.threshtype != 2) return {2.0 * fwd + sel, 0.0, 0.0};
  const double half = mod ? n * (d.J - 1) * 2.0 * L : n * 2.0 * L;  // both halves, one step
  const double steps = 40.0, terms = 4.0 * n, sum = 4.0 * n;
  const double pre = fwd + sel;
  const double solo = pre + fwd + steps * (half + terms + sum) + fwd;
  const double pair = pre + 0.5 * fwd + steps * (0.5 * half + 0.5 * terms + sum);
  return {solo, pair + fwd, pair};
}
double work_of(const BatchDesc& d) { return cost_of(d).solo; }

// Longest CTA busy time when the first npair CV candidates (cand, in
// decreasing work) run as pairs at the start and the remaining signals
// (byw, decreasing work) go one by one to the CTA that frees first: the
// queue's own schedule under the cost model.
double lpt_makespan(const std::vector<Cost>& cost, const std::vector<int>& byw,
                    const std::vector<int>& cand, int npair, int grid,
                    std::vector<char>& paired) {
  std::fill(paired.begin(), paired.end(), 0);
  std::vector<double> load;
  load.reserve(grid);
  for (int k = 0; k < npair; k++) {
    const Cost& c = cost[cand[k]];
    load.push_back(c.leader);
    load.push_back(c.partner);
    paired[cand[k]] = 1;
  }
  while ((int)load.size() < grid) load.push_back(0.0);
  std::make_heap(load.begin(), load.end(), std::greater<double>());
  for (int i : byw) {
    if (paired[i]) continue;
    std::pop_heap(load.begin(), load.end(), std::greater<double>());
    load.back() += cost[i].solo;
    std::push_heap(load.begin(), load.end(), std::greater<double>());
  }
  return *std::max_element(load.begin(), load.end());
}

// Whether the device runs a CV search for d (mirrors cv_runs and range_ok of
// the kernel: thresh.cpp:223-231 returns before searching otherwise).
bool cv_searches(const BatchDesc& d) {
  if (d.threshtype != 2 || d.J <= 1) return false;
  const int L = filter_len(d.F);
  int maxlev = 0;
  while (((int64_t)L << maxlev) <= d.n) maxlev++;
  if (d.J > maxlev || d.minl < 0 || d.maxl < 0) return false;
  return d.minl <= d.maxl && d.maxl < d.J;
}

void free_plan(wc_batch_plan_s* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  cudaFree(p->d_desc);
  cudaFree(p->d_res);
  cudaFree(p->d_order);
  cudaFree(p->d_counter);
  cudaFree(p->d_pairs);
  cudaFree(p->d_trace);
  if (p->own_scratch) cudaFree(p->d_scratch);
  delete p;
}

// Grid chosen by the last wc_batch_autotune per precision (0: none yet);
// later plans of the process start from it.
std::atomic<int> g_tuned_grid[3];

int launch_direct(wc_batch_plan_s* p, double* data, int grid, cudaStream_t s) {
  if (grid < 2 * p->npairs)
    return fail(WC_ERR_ARG, "grid %d below the %d CTAs of the paired searches", grid,
                2 * p->npairs);
  WC_CUDA(cudaMemsetAsync(p->d_counter, 0, sizeof(int), s));
  if (p->npairs > 0) WC_CUDA(cudaMemsetAsync(p->d_pairs, 0, sizeof(BatchPair) * p->npairs, s));
  BatchArgs a{p->d_desc,  p->d_res,         p->d_order, p->d_counter, p->nunits, data,
              p->d_scratch, p->scratch_per_cta, p->d_pairs, p->status,   p->d_trace};
  LaunchTimer lt("smooth_batch", s);
  return batch_launch(a, p->prec, grid, s);
}

}  // namespace
}  // namespace wc

using namespace wc;

extern "C" {

namespace wc {
namespace {
int plan_create(const wc_signal* sigs, int nsig, int precision, bool workspace_scratch,
                wc_batch_plan* out);
}  // namespace
}  // namespace wc

int wc_batch_plan_create(const wc_signal* sigs, int nsig, int precision, wc_batch_plan* out) {
  return wc::plan_create(sigs, nsig, precision, false, out);
}

}  // extern "C"

namespace wc {
namespace {

// workspace_scratch: the CTA scratch comes from the library's per-device
// workspace (kept between calls), for the synchronous host-buffer call.
int plan_create(const wc_signal* sigs, int nsig, int precision, bool workspace_scratch,
                wc_batch_plan* out) {
  clear_error();
  if (!sigs || nsig <= 0 || !out) return fail(WC_ERR_ARG, "bad batch arguments");
  if (precision < 0 || precision > 2) return fail(WC_ERR_ARG, "unknown precision %d", precision);
  WC_TRY(ensure_device());
  std::vector<BatchDesc> desc(nsig);
  int64_t total = 0;
  size_t per_cta = 0;
  for (int i = 0; i < nsig; i++) {
    const wc_signal& s = sigs[i];
    if (s.filter < 1 || s.filter > 4) return fail(WC_ERR_ARG, "signal %d: unrecognised filter", i);
    if (s.ttype != 0 && s.ttype != 1) return fail(WC_ERR_ARG, "signal %d: transform type", i);
    if (s.threshtype < 0 || s.threshtype > 2) return fail(WC_ERR_ARG, "signal %d: threshold type", i);
    if (s.offset < 0) return fail(WC_ERR_ARG, "signal %d: negative offset", i);
    const int L = filter_len(s.filter);
    const int J = check_levels(s.len, s.nlevels, L);
    if (J == 0) return fail(WC_ERR_LEVELS, "signal %d: nlevels %d invalid for length %lld", i,
                            s.nlevels, (long long)s.len);
    if (s.threshtype == 2 && !(s.tol > 0)) return fail(WC_ERR_ARG, "signal %d: tolerance", i);
    BatchDesc& d = desc[i];
    d.off = s.offset;
    d.n = s.len;
    d.J = J;
    d.ttype = s.ttype;
    d.F = s.filter;
    d.threshtype = s.threshtype;
    d.hardness = s.hardness;
    d.minl = s.minlevel;
    d.maxl = s.maxlevel;
    d.pair = 0;
    d.thresh = s.thresh;
    d.tol = s.tol;
    // thresh.cpp:180,198,326 evaluated with the host libm, as the reference does
    d.sq_n = sqrt(2. * log((double)s.len));
    d.sq_nm1 = sqrt(2. * log((double)(s.len - 1)));
    d.rescale = sqrt(1. - log(2.) / log((double)s.len));
    total = std::max(total, s.offset + s.len);
    per_cta = std::max(per_cta, batch_scratch_bytes(d, precision));
  }
  auto* p = new wc_batch_plan_s;
  p->nsig = nsig;
  p->prec = precision;
  p->total = total;
  p->scratch_per_cta = ((per_cta + 255) / 256) * 256;
  // Grid: every resident CTA, limited so that the CTA scratch takes at most
  // half of the free device memory.
  size_t freeb = 0, totb = 0;
  cudaMemGetInfo(&freeb, &totb);
  int grid = batch_max_ctas(precision);
  if (g_tuned_grid[precision].load() > 0) grid = std::min(grid, g_tuned_grid[precision].load());
  const size_t cap = (freeb / 2) / std::max<size_t>(p->scratch_per_cta, 1);
  grid = (int)std::min<size_t>((size_t)grid, std::max<size_t>(cap, 1));
  grid = std::min(grid, nsig);

  // Queue order, largest work first.  When a few long CV searches would
  // keep their CTAs busy after the rest of the batch is done, the longest of
  // them are split over two CTAs (a leader and a partner, one half-signal
  // inverse each per golden step): the number of pairs is the one whose
  // schedule under the cost model ends first, and pairing is used only when
  // that beats the unpaired schedule by 5 % (a pair does some work twice).
  // Paired units go first and number at most the grid, so each is taken by
  // some CTA's first pull: with every CTA resident, both CTAs of a pair
  // start together and neither waits on a CTA that is busy elsewhere.
  // WAVECUDA_BATCH_PAIRS=0 turns pairing off; =1 pairs every candidate
  // whose work is above half the even share per CTA (for tests).
  std::vector<int> byw(nsig);
  std::iota(byw.begin(), byw.end(), 0);
  std::stable_sort(byw.begin(), byw.end(),
                   [&](int a, int b) { return work_of(desc[a]) > work_of(desc[b]); });
  const char* pe = getenv("WAVECUDA_BATCH_PAIRS");
  const int pair_mode = (pe && pe[0] == '0') ? 0 : (pe && pe[0] == '1') ? 2 : 1;
  std::vector<int> cand;
  if (pair_mode != 0 && grid >= 2)
    for (int i : byw)
      if (cv_searches(desc[i]) && 2 * ((int)cand.size() + 1) <= grid) cand.push_back(i);
  int npairs = 0;
  if (!cand.empty()) {
    std::vector<char> paired(nsig, 0);
    if (pair_mode == 2) {
      double wsum = 0.0;
      for (int i = 0; i < nsig; i++) wsum += work_of(desc[i]);
      const double share = wsum / grid;
      while (npairs < (int)cand.size() && work_of(desc[cand[npairs]]) > 0.5 * share) npairs++;
    } else {
      std::vector<Cost> cost(nsig);
      for (int i = 0; i < nsig; i++) cost[i] = cost_of(desc[i]);
      const double m0 = lpt_makespan(cost, byw, cand, 0, grid, paired);
      double best = m0;
      int best_k = 0;
      for (int k = 1; k <= (int)cand.size(); k++) {
        const double m = lpt_makespan(cost, byw, cand, k, grid, paired);
        if (m < best) {
          best = m;
          best_k = k;
        }
      }
      npairs = (best < 0.95 * m0) ? best_k : 0;
    }
  }
  std::vector<int> order;
  order.reserve((size_t)nsig + npairs);
  for (int k = 0; k < npairs; k++) {
    desc[cand[k]].pair = k + 1;
    order.push_back(cand[k]);
    order.push_back(-(cand[k] + 1));
  }
  for (int i : byw)
    if (desc[i].pair == 0) order.push_back(i);
  p->npairs = npairs;
  p->nunits = (int)order.size();
  p->grid = grid;
  p->scratch_bytes = p->scratch_per_cta * (size_t)grid;
  cudaError_t e = cudaSuccess;
  if ((e = cudaMalloc(&p->d_desc, sizeof(BatchDesc) * nsig)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_res, sizeof(BatchResult) * nsig)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_order, sizeof(int) * p->nunits)) != cudaSuccess ||
      (npairs > 0 && (e = cudaMalloc(&p->d_pairs, sizeof(BatchPair) * npairs)) != cudaSuccess) ||
      (e = cudaMalloc(&p->d_counter, sizeof(int))) != cudaSuccess ||
      (!workspace_scratch && (e = cudaMalloc(&p->d_scratch, p->scratch_bytes)) != cudaSuccess)) {
    cudaGetLastError();
    free_plan(p);
    return fail(WC_ERR_NOMEM, "batch plan allocation failed: %s", cudaGetErrorString(e));
  }
  if (workspace_scratch) {
    p->own_scratch = false;
    p->d_scratch = static_cast<char*>(workspace(kSlotBatchScratch, p->scratch_bytes));
    if (!p->d_scratch) {
      free_plan(p);
      return workspace_error();
    }
  }
  cudaMemcpy(p->d_desc, desc.data(), sizeof(BatchDesc) * nsig, cudaMemcpyHostToDevice);
  cudaMemcpy(p->d_order, order.data(), sizeof(int) * p->nunits, cudaMemcpyHostToDevice);
  p->status = device_status_word();
  if (getenv("WAVECUDA_BATCH_TRACE")) {
    if (cudaMalloc(&p->d_trace, sizeof(unsigned long long) * 3 * (size_t)p->nunits) != cudaSuccess) {
      cudaGetLastError();
      p->d_trace = nullptr;
    } else {
      cudaMemset(p->d_trace, 0, sizeof(unsigned long long) * 3 * (size_t)p->nunits);
    }
    p->order = order;
    p->desc = desc;
  }
  cudaMemset(p->d_res, 0, sizeof(BatchResult) * nsig);
  *out = p;
  return WC_OK;
}

}  // namespace
}  // namespace wc

extern "C" {

int wc_batch_plan_destroy(wc_batch_plan plan) {
  free_plan(plan);
  return WC_OK;
}

int wc_batch_plan_info(wc_batch_plan plan, int* grid, size_t* scratch_bytes) {
  if (!plan) return fail(WC_ERR_ARG, "null plan");
  if (grid) *grid = plan->grid;
  if (scratch_bytes) *scratch_bytes = plan->scratch_bytes;
  return WC_OK;
}

int wc_batch_plan_pairs(wc_batch_plan plan, int* npairs) {
  if (!plan || !npairs) return fail(WC_ERR_ARG, "null plan or output");
  *npairs = plan->npairs;
  return WC_OK;
}

int wc_batch_run_device(wc_batch_plan plan, double* data, void* stream) {
  clear_error();
  if (!plan || !data) return fail(WC_ERR_ARG, "null plan or data");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  if (!plan->exec || plan->graph_data != data || plan->graph_stream != s ||
      plan->graph_grid != plan->grid) {
    if (plan->exec) {
      cudaGraphExecDestroy(plan->exec);
      plan->exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    cudaStream_t cap = nullptr;
    WC_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    WC_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    int r = launch_direct(plan, data, plan->grid, cap);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (r != WC_OK) return r;
    if (e != cudaSuccess) return fail(WC_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&plan->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(WC_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    plan->graph_data = data;
    plan->graph_stream = s;
    plan->graph_grid = plan->grid;
  }
  {
    LaunchTimer lt("smooth_batch_graph", s);
    WC_CUDA(cudaGraphLaunch(plan->exec, s));
  }
  count_launches(1);
  return WC_OK;
}

int wc_batch_results(wc_batch_plan plan, wc_signal_result* out, void* stream) {
  clear_error();
  if (!plan || !out) return fail(WC_ERR_ARG, "null plan or output");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lib_stream();
  std::vector<BatchResult> r(plan->nsig);
  WC_CUDA(cudaMemcpyAsync(r.data(), plan->d_res, sizeof(BatchResult) * plan->nsig,
                          cudaMemcpyDeviceToHost, s));
  WC_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < plan->nsig; i++) {
    out[i].thresh = r[i].thresh;
    out[i].thresh_univ = r[i].thresh_univ;
    out[i].min_margin = r[i].min_margin;
    out[i].iterations = r[i].iterations;
    out[i].status = r[i].status;
    out[i].kept = r[i].kept;
    out[i].zeroed = r[i].zeroed;
  }
  if (plan->d_trace) {
    // WAVECUDA_BATCH_TRACE=<path>: one CSV line per queue unit
    std::vector<unsigned long long> tr(3 * (size_t)plan->nunits);
    WC_CUDA(cudaMemcpy(tr.data(), plan->d_trace, sizeof(unsigned long long) * tr.size(),
                       cudaMemcpyDeviceToHost));
    if (FILE* f = fopen(getenv("WAVECUDA_BATCH_TRACE"), "w")) {
      fprintf(f, "unit,signal,role,n,filter,ttype,threshtype,start_ns,end_ns,cta\n");
      for (int k = 0; k < plan->nunits; k++) {
        const int u = plan->order[(size_t)k];
        const int i = u < 0 ? -u - 1 : u;
        const wc::BatchDesc& d = plan->desc[(size_t)i];
        const int role = u < 0 ? 2 : (d.pair > 0 ? 1 : 0);
        fprintf(f, "%d,%d,%d,%lld,%d,%d,%d,%llu,%llu,%llu\n", k, i, role, (long long)d.n, d.F,
                d.ttype, d.threshtype, tr[3 * (size_t)k], tr[3 * (size_t)k + 1],
                tr[3 * (size_t)k + 2]);
      }
      fclose(f);
    }
  }
  return WC_OK;
}

// Times the batch at a few grid sizes on a scratch copy of the data and keeps
// the fastest for the plan.  The data are not modified.
int wc_batch_autotune(wc_batch_plan plan, const double* data, float* best_ms) {
  clear_error();
  if (!plan || !data) return fail(WC_ERR_ARG, "null plan or data");
  cudaStream_t s = lib_stream();
  double* copy = nullptr;
  const size_t bytes = sizeof(double) * (size_t)plan->total;
  WC_CUDA(cudaMalloc(&copy, bytes));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  std::vector<int> cand = {plan->grid};
  for (int g : {sms / 2, sms, 2 * sms}) {
    if (g >= 1 && g < plan->grid && g >= 2 * plan->npairs) cand.push_back(g);
  }
  std::sort(cand.begin(), cand.end());
  cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int best_g = plan->grid;
  int rc = WC_OK;
  for (int g : cand) {
    cudaMemcpyAsync(copy, data, bytes, cudaMemcpyDeviceToDevice, s);
    cudaEventRecord(a, s);
    rc = launch_direct(plan, copy, g, s);
    cudaEventRecord(b, s);
    if (rc != WC_OK) break;
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) {
      best = ms;
      best_g = g;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(copy);
  if (rc != WC_OK) return rc;
  plan->grid = best_g;
  g_tuned_grid[plan->prec].store(best_g);
  if (best_ms) *best_ms = best;
  return WC_OK;
}

int wc_smooth_batch(double* data, int64_t total, const wc_signal* sigs, int nsig, int precision,
                    wc_signal_result* results) {
  clear_error();
  if (!data || !sigs || !results || total <= 0) return fail(WC_ERR_ARG, "bad batch arguments");
  for (int i = 0; i < nsig; i++)
    if (sigs[i].offset + sigs[i].len > total)
      return fail(WC_ERR_ARG, "signal %d extends past the data (%lld elements)", i, (long long)total);
  wc_batch_plan plan = nullptr;
  WC_TRY(wc::plan_create(sigs, nsig, precision, true, &plan));
  cudaStream_t s = lib_stream();
  double* d = static_cast<double*>(workspace(kSlotBatch, sizeof(double) * (size_t)total));
  int rc = d ? WC_OK : workspace_error();
  if (rc == WC_OK && cudaMemcpyAsync(d, data, sizeof(double) * (size_t)total,
                                     cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = fail(WC_ERR_CUDA, "copy to device failed");
  if (rc == WC_OK) rc = wc_batch_run_device(plan, d, s);
  if (rc == WC_OK) rc = take_status(s);  // data stay untouched when a wait gave up
  if (rc == WC_OK && cudaMemcpyAsync(data, d, sizeof(double) * (size_t)total,
                                     cudaMemcpyDeviceToHost, s) != cudaSuccess)
    rc = fail(WC_ERR_CUDA, "copy to host failed");
  if (rc == WC_OK) rc = wc_batch_results(plan, results, s);
  wc_batch_plan_destroy(plan);
  return rc;
}

}  // extern "C"
