// .C glue for R: status-returning forms of the reference's R-facing symbols
// and the flat batched smoothing entry point.
//
// R's .C interface passes every argument as a pointer to the first element of
// an R vector (double* for numeric, int* for integer) and copies the vectors
// back afterwards (rfunctions.R:345-356 of the reference); it cannot build C
// structs or pass scalars by value.  The wc_* calls take scalars by value and
// the batched call takes an array of wc_signal records, so these wrappers
// only unpack pointers, fill the records from parallel vectors and store the
// status code in an int the R side can test.  No computation happens here.
#include <stdint.h>
#include <stdlib.h>

#include <vector>

#include "wc_internal.h"

using namespace wc;

extern "C" {

void wc_transform_R(double* x, double* xmod, int* len, int* sense, int* nlevels, int* ttype,
                    int* filter, int* precision, int* status) {
  if (!status) return;
  if (!len || !sense || !nlevels || !ttype || !filter || !precision) {
    *status = WC_ERR_ARG;
    return;
  }
  *status = wc_transform(x, xmod, *len, *sense, *nlevels, *ttype, *filter, *precision);
}

void wc_threshold_R(double* x, double* xmod, int* len, int* nlevels, int* ttype, int* filter,
                    double* thresh, int* hardness, int* minlevel, int* maxlevel, int* status) {
  if (!status) return;
  if (!len || !nlevels || !ttype || !filter || !thresh || !hardness || !minlevel || !maxlevel) {
    *status = WC_ERR_ARG;
    return;
  }
  *status = wc_threshold(x, xmod, *len, *nlevels, *ttype, *filter, *thresh, *hardness, *minlevel,
                         *maxlevel);
}

void wc_smooth_R(double* x, int* len, int* nlevels, int* ttype, int* filter, int* threshtype,
                 double* thresh, int* hardness, int* minlevel, int* maxlevel, double* tol,
                 int* precision, int* status) {
  if (!status) return;
  if (!len || !nlevels || !ttype || !filter || !threshtype || !hardness || !minlevel ||
      !maxlevel || !tol || !precision) {
    *status = WC_ERR_ARG;
    return;
  }
  *status = wc_smooth(x, *len, *nlevels, *ttype, *filter, *threshtype, thresh, *hardness,
                      *minlevel, *maxlevel, *tol, *precision, nullptr);
}

// Batched smoothing in .C form: signal i occupies data[offset[i] ..
// offset[i] + len[i]) (0-based offsets) and is described by element i of the
// parallel vectors.  thresh[i] is the manual threshold on input and the
// threshold applied on output; iterations, kept and zeroed receive the CV
// iterations and the kept/zeroed detail counts per signal.  All signals are
// smoothed by one persistent launch (wc_smooth_batch).
void RgpuSmoothBatch(double* data, int* total, int* nsig, int* offset, int* len, int* nlevels,
                     int* ttype, int* filter, int* threshtype, double* thresh, int* hardness,
                     int* minlevel, int* maxlevel, double* tol, int* precision, int* iterations,
                     int* kept, int* zeroed, int* status) {
  if (!status) return;
  clear_error();
  if (!data || !total || !nsig || !offset || !len || !nlevels || !ttype || !filter ||
      !threshtype || !thresh || !hardness || !minlevel || !maxlevel || !tol || !precision) {
    *status = fail(WC_ERR_ARG, "null pointer among the batch vectors");
    return;
  }
  const int n = *nsig;
  if (n <= 0 || *total <= 0) {
    *status = fail(WC_ERR_ARG, "empty batch (nsig %d, total %d)", n, *total);
    return;
  }
  std::vector<wc_signal> sig((size_t)n);
  for (int i = 0; i < n; i++) {
    if (offset[i] < 0 || len[i] <= 0) {
      *status = fail(WC_ERR_ARG, "signal %d: offset %d / length %d invalid", i, offset[i], len[i]);
      return;
    }
    wc_signal& s = sig[(size_t)i];
    s.offset = offset[i];
    s.len = len[i];
    s.nlevels = nlevels[i];
    s.ttype = ttype[i];
    s.filter = filter[i];
    s.threshtype = threshtype[i];
    s.hardness = hardness[i];
    s.minlevel = minlevel[i];
    s.maxlevel = maxlevel[i];
    s.thresh = thresh[i];
    s.tol = tol[i];
  }
  std::vector<wc_signal_result> res((size_t)n);
  const int r = wc_smooth_batch(data, *total, sig.data(), n, *precision, res.data());
  *status = r;
  if (r != WC_OK) return;
  for (int i = 0; i < n; i++) {
    thresh[i] = res[(size_t)i].thresh;
    if (iterations) iterations[i] = res[(size_t)i].iterations;
    if (kept) kept[i] = (int)res[(size_t)i].kept;
    if (zeroed) zeroed[i] = (int)res[(size_t)i].zeroed;
  }
}

}  // extern "C"
