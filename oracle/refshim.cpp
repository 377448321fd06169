// Test infrastructure only (oracle).  Never linked into the product.
//
// CPU-only restatement of the R-facing entry points of the reference
// (rfunctions.cu:3-100: RcpuTransform, RcpuThreshold, RcpuSmooth) so that the
// reference's own CPU sources can be driven without R.  The wavelet work is
// done entirely by the reference functions this file calls: transform()
// (transform.cpp:3), threshold() (thresh.cpp:113), univ_thresh()
// (thresh.cpp:170), CVT() (thresh.cpp:203), median()/mad() (utils.cpp:166-203).
//
// Symbols are prefixed wref_ so that they never collide with the product's
// R-compatible symbols when both libraries are loaded into one process.

#include <cstdlib>
#include <cstring>
#include "transform.h"
#include "thresh.h"
#include "utils.h"

extern "C" {

// All reference allocations are routed here by the build (ref_zero_malloc.h):
// zero-filled, so reads of never-written slots are deterministic.
void* ref_zero_malloc(size_t n) { return calloc(n ? n : 1, 1); }

// rfunctions.cu:3-18 (RcpuTransform).  Returns the transform's status.
int wref_transform(double* x, double* xmod, int len, int sense, int nlevels,
                   int ttype, int filter, int filterlen) {
  wst* w = create_wvtstruct(x, xmod, (short)ttype, (short)filter,
                            (short)filterlen, (uint)nlevels, (uint)len);
  if (w == NULL) return 1;
  if (sense == BWD) w->transformed = 1;
  int res = transform(w, (short)sense);
  free(w);
  return res;
}

// rfunctions.cu:59-69 (RcpuThreshold).
int wref_threshold(double* x, double* xmod, int len, int nlevels, int ttype,
                   int filter, int filterlen, double thresh, int hardness,
                   int minlevel, int maxlevel) {
  wst* w = create_wvtstruct(x, xmod, (short)ttype, (short)filter,
                            (short)filterlen, (uint)nlevels, (uint)len);
  if (w == NULL) return 1;
  threshold(w, NULL, thresh, (short)hardness, (uint)minlevel, (uint)maxlevel);
  free(w);
  return 0;
}

// rfunctions.cu:71-100 (RcpuSmooth).  threshtype: 0 manual, 1 univ, 2 cv.
// *thresh is input for manual and output for univ/cv, as in the reference.
// For MODWT the reference allocates xmod inside create_wvtstruct
// (wavutils.cpp:611-623); it is released here (the reference leaks it).
int wref_smooth(double* x, int len, int nlevels, int ttype, int filter,
                int filterlen, int threshtype, double* thresh, int hardness,
                int minlevel, int maxlevel, double tol) {
  wst* w = create_wvtstruct(x, (short)ttype, (short)filter, (short)filterlen,
                            (uint)nlevels, (uint)len);
  if (w == NULL) return 1;
  switch (threshtype) {
    case 2:
      *thresh = CVT(w, (short)hardness, tol, (uint)minlevel, (uint)maxlevel);
      break;
    case 1:
      transform(w, FWD);
      *thresh = univ_thresh(w, 0, 0);
      threshold(w, NULL, *thresh, (short)hardness, (uint)minlevel, (uint)maxlevel);
      transform(w, BWD);
      break;
    case 0:
      transform(w, FWD);
      threshold(w, NULL, *thresh, (short)hardness, (uint)minlevel, (uint)maxlevel);
      transform(w, BWD);
      break;
    default:
      free(w);
      return 2;
  }
  if (w->ttype == MODWT_TO || w->ttype == MODWT_PO) free(w->xmod);
  free(w);
  return 0;
}

// univ_thresh (thresh.cpp:170-201) on an already transformed vector.
double wref_univ_thresh(double* x, double* xmod, int len, int nlevels,
                        int ttype, int filter, int filterlen, int minlevel,
                        int maxlevel) {
  wst* w = create_wvtstruct(x, xmod, (short)ttype, (short)filter,
                            (short)filterlen, (uint)nlevels, (uint)len);
  if (w == NULL) return -1.0;
  w->transformed = 1;
  double t = univ_thresh(w, (uint)minlevel, (uint)maxlevel);
  free(w);
  return t;
}

// median / mad (utils.cpp:166-203).
double wref_median(double* x, int len) { return median(x, (uint)len); }
double wref_mad(double* x, int len) { return mad(x, (uint)len); }

// check_len_levels (wavutils.cpp:48-64).
unsigned wref_check_len_levels(unsigned len, unsigned nlevels, unsigned filterlength) {
  return check_len_levels(len, nlevels, filterlength);
}

}  // extern "C"
