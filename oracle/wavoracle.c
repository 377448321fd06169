/*
 * wavoracle.c -- CPU restatement of the wavecuda reference's FP64 CPU path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline; the product library
 * never links or calls it.
 *
 * Arithmetic is written so that every result is bit-identical to the
 * reference CPU code built without FMA contraction: the same literal filter
 * constants (haarcoeffs.h:4-5, daub4coeffs.h:13-16, c6coeffs.h:6-11,
 * la8coeffs.h:6-13) and the same left-to-right order of products and sums as
 * the reference expressions cited at each function.  Subtractions of a
 * product in the reference (a - x*C) are written as additions of x*(-C),
 * which rounds identically.  Indices are 64-bit.
 *
 * The per-level transform loops run on OpenMP threads for long levels.  Each
 * output of a level depends only on the previous level, so the thread count
 * changes no result; wo_set_threads(1) gives the reference's serial loop.
 */
#include "wavoracle.h"

#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define WO_FWD 1
#define WO_BWD 0
#define WO_HAAR 1
#define WO_D4 2
#define WO_C6 3
#define WO_LA8 4
#define WO_DWT 0
#define WO_MODWT 1
#define WO_MODWT_PO 2
#define WO_HARD 0
#define WO_SOFT 1

static const double kInvR2 = 0.70710678118654752440;  /* haarcoeffs.h:4 */
static const double kHInvR2 = 0.35355339059327376220; /* haarcoeffs.h:5 */

static const double kD4[4] = {0.4829629131445341, 0.8365163037378079,
                              0.2241438680420134, -0.1294095225512604};
static const double kC6[6] = {-7.273261951252645e-2, 3.378976624574818e-1,
                              8.525720202116004e-1,  3.848648468648577e-1,
                              -7.273261951252645e-2, -1.565572813579199e-2};
static const double kLA8[8] = {-7.576571478950221e-2, -2.963552764600249e-2,
                               4.976186676327750e-1,  8.037387518051321e-1,
                               2.978577956053061e-1,  -9.921954357663353e-2,
                               -1.260396726203130e-2, 3.222310060405147e-2};

int wo_filter_length(int filter) {
  switch (filter) {
    case WO_HAAR: return 2;
    case WO_D4: return 4;
    case WO_C6: return 6;
    case WO_LA8: return 8;
    default: return 0;
  }
}

/* Scaling taps h_k and wavelet taps g_k = (-1)^k h_{L-1-k}. */
static int get_taps(int filter, double* h, double* g) {
  const double* c = NULL;
  int L = wo_filter_length(filter);
  switch (filter) {
    case WO_HAAR: h[0] = h[1] = kInvR2; g[0] = kInvR2; g[1] = -kInvR2; return 2;
    case WO_D4: c = kD4; break;
    case WO_C6: c = kC6; break;
    case WO_LA8: c = kLA8; break;
    default: return 0;
  }
  for (int k = 0; k < L; k++) {
    h[k] = c[k];
    g[k] = (k & 1) ? -c[L - 1 - k] : c[L - 1 - k];
  }
  return L;
}

/* Levels shorter than this run serially. */
#define WO_PAR_MIN 32768

void wo_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
  (void)n;
#endif
}

int wo_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int is_pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

/* wavutils.cpp:48-64 */
int wo_check_len_levels(int64_t len, int nlevels, int filterlen) {
  if (!is_pow2(len) || filterlen <= 0) return 0;
  if (len < filterlen) return 0;
  int maxlevels = (int)floor(log2((double)len / filterlen)) + 1;
  if (nlevels == 0) nlevels = maxlevels;
  if (nlevels < 0 || nlevels > maxlevels) return 0;
  return nlevels;
}

/* wavutils.cpp:66-77 */
static int check_levels_range(int64_t len, int nlevels, int minlevel,
                              int maxlevel, int filterlen) {
  int ret = wo_check_len_levels(len, nlevels, filterlen);
  if (ret == 0) return 0;
  if (minlevel < 0 || maxlevel < 0) return 0; /* uint wrap in the reference */
  if (minlevel > maxlevel || maxlevel >= ret) return 0;
  return ret;
}

/* ------------------------------------------------------------------ DWT -- */

/* One forward level on the subsequence y[m] = x[m*skip], m < N (conv form,
 * daub4.cpp:20-54, c6.cpp:32-75, la8.cpp:27-75; Haar haar.cpp:47-74). */
static void dwt_fwd_level(double* x, int64_t len, int64_t skip, int filter,
                          double* tmp) {
  const int64_t N = len / skip;
#pragma omp parallel for if (N >= WO_PAR_MIN) schedule(static)
  for (int64_t m = 0; m < N; m++) tmp[m] = x[m * skip];
  if (filter == WO_HAAR) {
#pragma omp parallel for if (N >= WO_PAR_MIN) schedule(static)
    for (int64_t q = 0; q < N / 2; q++) {
      double a = tmp[2 * q], b = tmp[2 * q + 1];
      x[(2 * q + 1) * skip] = (a - b) * kInvR2;
      x[(2 * q) * skip] = (a + b) * kInvR2;
    }
    return;
  }
  double h[8], g[8];
  int L = get_taps(filter, h, g);
#pragma omp parallel for if (N >= WO_PAR_MIN) schedule(static)
  for (int64_t q = 0; q < N / 2; q++) {
    double s = tmp[(2 * q) % N] * h[0];
    double d = tmp[(2 * q) % N] * g[0];
    for (int k = 1; k < L; k++) {
      double v = tmp[(2 * q + k) % N];
      s = s + v * h[k];
      d = d + v * g[k];
    }
    x[(2 * q) * skip] = s;
    x[(2 * q + 1) * skip] = d;
  }
}

/* One inverse level (daub4.cpp:58-88, c6.cpp:78-111, la8.cpp:79-115):
 * x_even[q] = sum_{j desc} h_{2j} s[q-j] + g_{2j} d[q-j],
 * x_odd[q]  = sum_{j desc} h_{2j+1} s[q-j] + g_{2j+1} d[q-j]. */
static void dwt_inv_level(double* x, int64_t len, int64_t skip, int filter,
                          double* tmp) {
  const int64_t N = len / skip, P = N / 2;
#pragma omp parallel for if (N >= WO_PAR_MIN) schedule(static)
  for (int64_t m = 0; m < N; m++) tmp[m] = x[m * skip];
  if (filter == WO_HAAR) {
#pragma omp parallel for if (N >= WO_PAR_MIN) schedule(static)
    for (int64_t q = 0; q < P; q++) {
      double a = tmp[2 * q], b = tmp[2 * q + 1];
      x[(2 * q + 1) * skip] = (a - b) * kInvR2;
      x[(2 * q) * skip] = (a + b) * kInvR2;
    }
    return;
  }
  double h[8], g[8];
  int L = get_taps(filter, h, g);
  const int H = L / 2;
#pragma omp parallel for if (N >= WO_PAR_MIN) schedule(static)
  for (int64_t q = 0; q < P; q++) {
    double e = 0.0, o = 0.0;
    for (int j = H - 1; j >= 0; j--) {
      int64_t p = ((q - j) % P + P) % P;
      double sv = tmp[2 * p], dv = tmp[2 * p + 1];
      if (j == H - 1) {
        e = sv * h[2 * j];
        o = sv * h[2 * j + 1];
      } else {
        e = e + sv * h[2 * j];
        o = o + sv * h[2 * j + 1];
      }
      e = e + dv * g[2 * j];
      o = o + dv * g[2 * j + 1];
    }
    x[(2 * q) * skip] = e;
    x[(2 * q + 1) * skip] = o;
  }
}

int wo_dwt(double* x, int64_t len, int sense, int nlevels, int filter) {
  int L = wo_filter_length(filter);
  if (L == 0) return 1;
  int J = wo_check_len_levels(len, nlevels, L);
  if (J == 0) return 1;
  double* tmp = (double*)malloc((size_t)len * sizeof(double));
  if (!tmp) return 1;
  if (sense == WO_FWD) {
    for (int l = 0; l < J; l++) dwt_fwd_level(x, len, (int64_t)1 << l, filter, tmp);
  } else if (sense == WO_BWD) {
    for (int l = J - 1; l >= 0; l--) dwt_inv_level(x, len, (int64_t)1 << l, filter, tmp);
  } else {
    free(tmp);
    return 1;
  }
  free(tmp);
  return 0;
}

/* ---------------------------------------------------------------- MODWT -- */

/* fHaarSDout (haar.cpp:590-600) / fDaub4SDout (daub4.cpp:561-571),
 * generalised to L taps. */
static void modwt_fwd_level(const double* X, double* S, double* D, int64_t len,
                            int64_t skip, int filter) {
  const int64_t mask = len - 1;
  if (filter == WO_HAAR) {
#pragma omp parallel for if (len >= WO_PAR_MIN) schedule(static)
    for (int64_t i = 0; i < len; i++) {
      double a = X[i], b = X[(i + skip) & mask];
      D[i] = (a - b) * kInvR2;
      S[i] = (a + b) * kInvR2;
    }
    return;
  }
  double h[8], g[8];
  int L = get_taps(filter, h, g);
#pragma omp parallel for if (len >= WO_PAR_MIN) schedule(static)
  for (int64_t i = 0; i < len; i++) {
    double v = X[i];
    double d = v * g[0], s = v * h[0];
    for (int k = 1; k < L; k++) {
      v = X[(i + (int64_t)k * skip) & mask];
      d = d + v * g[k];
      s = s + v * h[k];
    }
    D[i] = d;
    S[i] = s;
  }
}

/* bHaarSDout (haar.cpp:602-616) / bDaub4SDout (daub4.cpp:573-589),
 * generalised: 0.5 * (even taps descending, then odd taps descending), each
 * tap contributing h_k*S then g_k*D at i - k*skip. */
static void modwt_inv_level(double* Xout, const double* S, const double* D,
                            int64_t len, int64_t skip, int filter) {
  const int64_t mask = len - 1;
  if (filter == WO_HAAR) {
#pragma omp parallel for if (len >= WO_PAR_MIN) schedule(static)
    for (int64_t i = 0; i < len; i++) {
      int64_t j = (i - skip) & mask;
      Xout[i] = (S[i] + D[i] + S[j] - D[j]) * kHInvR2;
    }
    return;
  }
  double h[8], g[8];
  int L = get_taps(filter, h, g);
  int order[8], n = 0;
  for (int k = L - 2; k >= 0; k -= 2) order[n++] = k;
  for (int k = L - 1; k >= 1; k -= 2) order[n++] = k;
#pragma omp parallel for if (len >= WO_PAR_MIN) schedule(static)
  for (int64_t i = 0; i < len; i++) {
    double acc = 0.0;
    for (int t = 0; t < L; t++) {
      int k = order[t];
      int64_t j = (i - (int64_t)k * skip) & mask;
      if (t == 0) acc = S[j] * h[k];
      else acc = acc + S[j] * h[k];
      acc = acc + D[j] * g[k];
    }
    Xout[i] = 0.5 * acc;
  }
}

int wo_modwt(double* x, double* xmod, int64_t len, int sense, int nlevels,
             int filter) {
  int L = wo_filter_length(filter);
  if (L == 0) return 1;
  int J = wo_check_len_levels(len, nlevels, L);
  if (J == 0) return 1;
  if (sense == WO_FWD) {
    for (int l = 0; l < J; l++) {
      const double* X = (l == 0) ? x : xmod + (int64_t)2 * (l - 1) * len;
      modwt_fwd_level(X, xmod + (int64_t)2 * l * len,
                      xmod + (int64_t)(2 * l + 1) * len, len, (int64_t)1 << l,
                      filter);
    }
  } else if (sense == WO_BWD) {
    for (int l = J - 1; l >= 0; l--) {
      double* out = (l == 0) ? x : xmod + (int64_t)2 * (l - 1) * len;
      modwt_inv_level(out, xmod + (int64_t)2 * l * len,
                      xmod + (int64_t)(2 * l + 1) * len, len, (int64_t)1 << l,
                      filter);
    }
  } else {
    return 1;
  }
  return 0;
}

/* ------------------------------------------------- packet-ordered MODWT -- */

/* Reverses the low nb bits of v (reverse_bits, utils.cpp:254). */
static int64_t rev_bits(int64_t v, int nb) {
  int64_t r = 0;
  for (int i = 0; i < nb; i++) r = (r << 1) | ((v >> i) & 1);
  return r;
}

/* Level l of the packet-ordered layout from the time-ordered one
 * (convert_modwt_level, wavutils.cpp:569-600): packet `sh` holds the (s, d)
 * pairs of time positions t = rev(sh, l+1) + 2^(l+1) k, interleaved. */
static void to_to_po_level(const double* to, double* po, int64_t len, int l) {
  const int64_t skip = (int64_t)1 << l, lenos = len / skip, np = 2 * skip;
  for (int64_t sh = 0; sh < np; sh++) {
    const int64_t st = rev_bits(sh, l + 1);
    for (int64_t k = 0; k < lenos / 2; k++) {
      po[sh * lenos + 2 * k] = to[st + 2 * skip * k];
      po[sh * lenos + 2 * k + 1] = to[len + st + 2 * skip * k];
    }
  }
}

static void po_to_to_level(const double* po, double* to, int64_t len, int l) {
  const int64_t skip = (int64_t)1 << l, lenos = len / skip, np = 2 * skip;
  for (int64_t sh = 0; sh < np; sh++) {
    const int64_t st = rev_bits(sh, l + 1);
    for (int64_t k = 0; k < lenos / 2; k++) {
      to[st + 2 * skip * k] = po[sh * lenos + 2 * k];
      to[len + st + 2 * skip * k] = po[sh * lenos + 2 * k + 1];
    }
  }
}

/* One value of the one-level inverse DWT of a packet (bHaar / bDaub4 / ...
 * on lenos values, as dwt_inv_level) at packet position i; the packet's
 * pairs are (S, D)[r + 2 skip q], q < P. */
static double po_packet_inv(const double* S, const double* D, int64_t r, int64_t skip,
                            int64_t P, int64_t i, int filter, const double* h,
                            const double* g) {
  const int64_t q = i >> 1;
  const int odd = (int)(i & 1);
  if (filter == WO_HAAR) {
    const double a = S[r + 2 * skip * q], b = D[r + 2 * skip * q];
    return odd ? (a - b) * kInvR2 : (a + b) * kInvR2;
  }
  const int H = wo_filter_length(filter) / 2;
  double acc = 0.0;
  for (int j = H - 1; j >= 0; j--) {
    const int64_t p = ((q - j) % P + P) % P;
    const double sv = S[r + 2 * skip * p], dv = D[r + 2 * skip * p];
    if (j == H - 1) acc = sv * h[2 * j + odd];
    else acc = acc + sv * h[2 * j + odd];
    acc = acc + dv * g[2 * j + odd];
  }
  return acc;
}

/* Inverse of level l (bHaarMODWT, haar.cpp:363-398; bDaub4MODWTpo,
 * daub4.cpp:449-484): every packet pair (2m, 2m+1) is inverted one DWT level
 * and the two reconstructions are averaged, writeavpackets
 * (wavutils.cpp:304-330): out = 0.5 * (y_2m[i] + y_2m+1[(i - 1) mod lenos]).
 * In time order, packet 2m has residue st = u mod skip and packet 2m+1
 * residue st + skip (mod 2 skip); u = st + skip i. */
static void po_inv_level(const double* S, const double* D, double* out, int64_t len, int l,
                         int filter) {
  double h[8], g[8];
  get_taps(filter, h, g);
  const int64_t skip = (int64_t)1 << l, lenos = len / skip, P = lenos / 2;
  for (int64_t u = 0; u < len; u++) {
    const int64_t st = u % skip, i = u / skip;
    const double a = po_packet_inv(S, D, st, skip, P, i, filter, h, g);
    const double b = po_packet_inv(S, D, st + skip, skip, P, (i + lenos - 1) % lenos, filter,
                                   h, g);
    out[u] = 0.5 * (a + b);
  }
}

int wo_modwt_po(double* x, double* xmod, int64_t len, int sense, int nlevels, int filter) {
  int L = wo_filter_length(filter);
  if (L == 0) return 1;
  int J = wo_check_len_levels(len, nlevels, L);
  if (J == 0) return 1;
  double* to = (double*)malloc(sizeof(double) * (size_t)(2 * (int64_t)J * len));
  if (!to) return 1;
  if (sense == WO_FWD) {
    /* fHaarMODWT / fDaub4MODWTpo compute the same coefficients as the
     * time-ordered transform, stored per packet. */
    wo_modwt(x, to, len, WO_FWD, J, filter);
    for (int l = 0; l < J; l++)
      to_to_po_level(to + 2 * (int64_t)l * len, xmod + 2 * (int64_t)l * len, len, l);
  } else if (sense == WO_BWD) {
    for (int l = 0; l < J; l++)
      po_to_to_level(xmod + 2 * (int64_t)l * len, to + 2 * (int64_t)l * len, len, l);
    double* cur = (double*)malloc(sizeof(double) * (size_t)len);
    double* nxt = (double*)malloc(sizeof(double) * (size_t)len);
    if (!cur || !nxt) {
      free(cur); free(nxt); free(to);
      return 1;
    }
    memcpy(cur, to + 2 * (int64_t)(J - 1) * len, sizeof(double) * (size_t)len);
    for (int l = J - 1; l >= 0; l--) {
      double* dst = (l == 0) ? x : nxt;
      po_inv_level(cur, to + (2 * (int64_t)l + 1) * len, dst, len, l, filter);
      double* t = cur; cur = nxt; nxt = t;
    }
    free(cur);
    free(nxt);
  } else {
    free(to);
    return 1;
  }
  free(to);
  return 0;
}

/* ----------------------------------------------------------- threshold -- */

double wo_thresh_coef(double coef, double thresh, int hardness) {
  if (fabs(coef) < thresh) return 0.0;
  if (hardness == WO_SOFT) return ((coef < 0) ? -1 : 1) * (fabs(coef) - thresh);
  return coef;
}

/* threshold_dwt with level limits (thresh.cpp:15-35).  out == NULL: in place.
 * Otherwise out[0] and every detail slot are written; the coarse scaling
 * slots k*2^levels (k > 0) are written only when copy_scaling is set. */
static void threshold_dwt(const double* in, double* out, int64_t len,
                          double thresh, int hardness, int minlevel,
                          int maxlevel, int levels, int copy_scaling) {
  int inplace = (out == NULL);
  if (inplace) out = (double*)in;
  else out[0] = in[0];
  for (int l = 0; l < levels; l++) {
    int64_t skip = (int64_t)1 << l;
    int in_range = (l >= minlevel) && (l <= maxlevel);
    for (int64_t i = skip; i < len; i += 2 * skip) {
      if (in_range) out[i] = wo_thresh_coef(in[i], thresh, hardness);
      else if (!inplace) out[i] = in[i];
    }
  }
  if (!inplace && copy_scaling) {
    int64_t step = (int64_t)1 << levels;
    for (int64_t i = step; i < len; i += step) out[i] = in[i];
  }
}

/* threshold_modwt, time ordered (thresh.cpp:41-83). */
static void threshold_modwt(const double* in, double* out, int64_t len,
                            double thresh, int hardness, int minlevel,
                            int maxlevel, int levels) {
  int inplace = (out == NULL);
  if (inplace) out = (double*)in;
  for (int l = 0; l < levels; l++) {
    int64_t il = (int64_t)2 * l * len;
    int in_range = (l >= minlevel) && (l <= maxlevel);
    for (int64_t i = 0; i < 2 * len; i++) {
      if (in_range && i >= len) out[il + i] = wo_thresh_coef(in[il + i], thresh, hardness);
      else if (!inplace) out[il + i] = in[il + i];
    }
  }
}

/* Packet order: the details sit at the odd indices of each level block
 * (thresh.cpp:56-64). */
static void threshold_modwt_po(double* xm, int64_t len, double thresh, int hardness,
                               int minlevel, int maxlevel) {
  for (int l = minlevel; l <= maxlevel; l++) {
    int64_t il = (int64_t)2 * l * len;
    for (int64_t i = 1; i < 2 * len; i += 2)
      xm[il + i] = wo_thresh_coef(xm[il + i], thresh, hardness);
  }
}

int wo_threshold(double* x, double* xmod, int64_t len, int nlevels, int ttype,
                 int filter, double thresh, int hardness, int minlevel,
                 int maxlevel) {
  int L = wo_filter_length(filter);
  if (check_levels_range(len, nlevels, minlevel, maxlevel, L) == 0) return 1;
  if (ttype == WO_DWT)
    threshold_dwt(x, NULL, len, thresh, hardness, minlevel, maxlevel, nlevels, 0);
  else if (ttype == WO_MODWT)
    threshold_modwt(xmod, NULL, len, thresh, hardness, minlevel, maxlevel, nlevels);
  else if (ttype == WO_MODWT_PO)
    threshold_modwt_po(xmod, len, thresh, hardness, minlevel, maxlevel);
  else
    return 1;
  return 0;
}

/* ---------------------------------------------------------- median/MAD -- */

static int cmp_double(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return (x < y) ? -1 : (x > y) ? 1 : 0;
}

/* utils.cpp:170-189: 0.5*(a[(n-1)/2] + a[n/2]) of the sorted copy. */
double wo_median(const double* x, int64_t len) {
  if (len <= 0) return 0.0;
  double* t = (double*)malloc((size_t)len * sizeof(double));
  memcpy(t, x, (size_t)len * sizeof(double));
  qsort(t, (size_t)len, sizeof(double), cmp_double);
  double m = 0.5 * (t[(len - 1) / 2] + t[len / 2]);
  free(t);
  return m;
}

/* utils.cpp:191-203 */
double wo_mad(const double* x, int64_t len) {
  if (len <= 0) return 0.0;
  double med = wo_median(x, len);
  double* dev = (double*)malloc((size_t)len * sizeof(double));
  for (int64_t i = 0; i < len; i++) dev[i] = fabs(x[i] - med);
  double m = wo_median(dev, len);
  free(dev);
  return 1.4826 * m;
}

/* thresh.cpp:170-201 with isolate_dlevels (wavutils.cpp:683-732). */
double wo_univ_thresh(const double* x, const double* xmod, int64_t len,
                      int nlevels, int ttype, int minlevel, int maxlevel) {
  int64_t n = 0;
  double* tmp;
  if (ttype == WO_DWT) {
    if (minlevel == 0 && maxlevel == nlevels - 1)
      return wo_mad(x + 1, len - 1) * sqrt(2. * log((double)(len - 1)));
    for (int l = minlevel; l <= maxlevel; l++) n += len >> (l + 1);
    tmp = (double*)malloc((size_t)(n ? n : 1) * sizeof(double));
    int64_t j = 0;
    for (int l = 0; l < nlevels; l++) {
      if (l < minlevel || l > maxlevel) continue;
      int64_t skip = (int64_t)1 << l;
      for (int64_t i = skip; i < len; i += 2 * skip) tmp[j++] = x[i];
    }
  } else if (ttype == WO_MODWT) {
    /* isolate_dlevels for the time-ordered layout (wavutils.cpp:716-722)
     * starts copying at the level-0 detail block whatever minlevel is, so it
     * gathers levels 0 .. maxlevel-minlevel. */
    n = (int64_t)(maxlevel - minlevel + 1) * len;
    tmp = (double*)malloc((size_t)(n ? n : 1) * sizeof(double));
    for (int l = 0; l <= maxlevel - minlevel; l++)
      memcpy(tmp + (int64_t)l * len, xmod + (int64_t)(2 * l + 1) * len,
             (size_t)len * sizeof(double));
  } else {
    return 0.0;
  }
  double ut = wo_mad(tmp, n) * sqrt(2. * log((double)len));
  free(tmp);
  return ut;
}

/* thresh.cpp:344-385 */
double wo_interp_mse(const double* xn, const double* ye, const double* yo,
                     int64_t len) {
  const int64_t lenh = len / 2;
  double m = 0.0, yie, yio;
  int64_t j = 0;
  for (int64_t i = 0; i < len; i += 2) {
    if (i == 0) {
      yie = yo[0];
      yio = 0.5 * (ye[j] + ye[j + 1]);
    } else if (i == len - 2) {
      yio = ye[lenh - 1];
      yie = 0.5 * (yo[j] + yo[j - 1]);
    } else {
      yio = 0.5 * (ye[j] + ye[j + 1]);
      yie = 0.5 * (yo[j] + yo[j - 1]);
    }
    j++;
    m += (yie - xn[i]) * (yie - xn[i]) + (yio - xn[i + 1]) * (yio - xn[i + 1]);
  }
  return m * 0.5;
}

/* ------------------------------------------------------------------ CVT -- */

typedef struct {
  double* x;    /* len doubles */
  double* xmod; /* 2*len*levels doubles (MODWT) or NULL */
  int transformed;
} wo_vec;

static int vec_alloc(wo_vec* v, int64_t len, int levels, int ttype) {
  v->x = (double*)calloc((size_t)len, sizeof(double));
  v->xmod = NULL;
  v->transformed = 0;
  if (ttype == WO_MODWT)
    v->xmod = (double*)calloc((size_t)(2 * len * levels), sizeof(double));
  return v->x != NULL && (ttype != WO_MODWT || v->xmod != NULL);
}

static void vec_free(wo_vec* v) {
  free(v->x);
  free(v->xmod);
}

/* transform() (transform.cpp:3-77): refuses to go in the direction the
 * vector is already in, and toggles the flag otherwise. */
static int vec_transform(wo_vec* v, int64_t len, int levels, int ttype,
                         int filter, int sense) {
  if (sense == v->transformed) return 1;
  int r = (ttype == WO_DWT) ? wo_dwt(v->x, len, sense, levels, filter)
                            : wo_modwt(v->x, v->xmod, len, sense, levels, filter);
  v->transformed = !v->transformed;
  return r;
}

/* threshold(win, wout, ...) with level limits (thresh.cpp:113-140). */
static void vec_threshold_to(const wo_vec* in, wo_vec* out, int64_t len,
                             int levels, int ttype, int filter, double t,
                             int hardness, int minlevel, int maxlevel,
                             int copy_scaling) {
  int L = wo_filter_length(filter);
  if (check_levels_range(len, levels, minlevel, maxlevel, L) == 0) return;
  if (ttype == WO_DWT)
    threshold_dwt(in->x, out->x, len, t, hardness, minlevel, maxlevel, levels,
                  copy_scaling);
  else
    threshold_modwt(in->xmod, out->xmod, len, t, hardness, minlevel, maxlevel,
                    levels);
  out->transformed = 1;
}

double wo_cvt(double* x, int64_t len, int nlevels, int ttype, int filter,
              int hardness, double tol, int minlevel, int maxlevel,
              int dwt_copy_scaling, wo_cv_trace* trace) {
  const double R = 0.61803399, C = 1. - R;
  int L = wo_filter_length(filter);
  int levels = wo_check_len_levels(len, nlevels, L);
  if (trace) memset(trace, 0, sizeof(*trace));
  if (levels == 0) return 0.0;
  if (check_levels_range(len, levels, minlevel, maxlevel, L) == 0) return 0.0;
  if (levels <= 1) return 0.0;
  const int64_t lenh = len >> 1;
  const int lv1 = levels - 1;
  wo_vec y1e, y1o, y2e, y2o, we, wo, w;
  vec_alloc(&y1e, lenh, lv1, ttype);
  vec_alloc(&y1o, lenh, lv1, ttype);
  vec_alloc(&y2e, lenh, lv1, ttype);
  vec_alloc(&y2o, lenh, lv1, ttype);
  vec_alloc(&we, lenh, lv1, ttype);
  vec_alloc(&wo, lenh, lv1, ttype);
  for (int64_t i = 0; i < lenh; i++) {
    we.x[i] = x[2 * i];
    wo.x[i] = x[2 * i + 1];
  }
  double* xn = (double*)malloc((size_t)len * sizeof(double));
  memcpy(xn, x, (size_t)len * sizeof(double));
  w.x = x;
  w.xmod = (ttype == WO_MODWT)
               ? (double*)calloc((size_t)(2 * len * levels), sizeof(double))
               : NULL;
  w.transformed = 0;
  vec_transform(&w, len, levels, ttype, filter, WO_FWD);
  double ta = 0., tc = wo_univ_thresh(w.x, w.xmod, len, levels, ttype, minlevel,
                                      maxlevel);
  if (trace) trace->t_univ = tc;
  double tb = tc / 2.;
  double t0 = ta, t2 = tb, t1 = tb - C * (tb - ta), t3 = tc;
  /* maxlevel - 1 in uint arithmetic wraps when maxlevel == 0; the range check
   * then fails and the half-length vectors are never thresholded. */
  int maxlevel1 = maxlevel - 1;
  vec_transform(&we, lenh, lv1, ttype, filter, WO_FWD);
  vec_transform(&wo, lenh, lv1, ttype, filter, WO_FWD);
  vec_threshold_to(&we, &y1e, lenh, lv1, ttype, filter, t1, hardness, minlevel, maxlevel1, dwt_copy_scaling);
  vec_threshold_to(&wo, &y1o, lenh, lv1, ttype, filter, t1, hardness, minlevel, maxlevel1, dwt_copy_scaling);
  vec_threshold_to(&we, &y2e, lenh, lv1, ttype, filter, t2, hardness, minlevel, maxlevel1, dwt_copy_scaling);
  vec_threshold_to(&wo, &y2o, lenh, lv1, ttype, filter, t2, hardness, minlevel, maxlevel1, dwt_copy_scaling);
  vec_transform(&y1e, lenh, lv1, ttype, filter, WO_BWD);
  vec_transform(&y1o, lenh, lv1, ttype, filter, WO_BWD);
  vec_transform(&y2e, lenh, lv1, ttype, filter, WO_BWD);
  vec_transform(&y2o, lenh, lv1, ttype, filter, WO_BWD);
  double m1 = wo_interp_mse(xn, y1e.x, y1o.x, len);
  double m2 = wo_interp_mse(xn, y2e.x, y2o.x, len);
  int iter = 0;
  while (fabs(t3 - t0) > tol * (t1 + t2)) {
    if (iter > 50) break;
    if (trace && iter < 64) {
      trace->t1[iter] = t1; trace->t2[iter] = t2;
      trace->m1[iter] = m1; trace->m2[iter] = m2;
      trace->took_m2[iter] = (m2 < m1);
    }
    if (m2 < m1) {
      t0 = t1; t1 = t2; t2 = R * t2 + C * t3;
      m1 = m2;
      vec_threshold_to(&we, &y2e, lenh, lv1, ttype, filter, t2, hardness, minlevel, maxlevel1, dwt_copy_scaling);
      vec_threshold_to(&wo, &y2o, lenh, lv1, ttype, filter, t2, hardness, minlevel, maxlevel1, dwt_copy_scaling);
      vec_transform(&y2e, lenh, lv1, ttype, filter, WO_BWD);
      vec_transform(&y2o, lenh, lv1, ttype, filter, WO_BWD);
      m2 = wo_interp_mse(xn, y2e.x, y2o.x, len);
    } else {
      t3 = t2; t2 = t1; t1 = R * t1 + C * t0;
      m2 = m1;
      vec_threshold_to(&we, &y1e, lenh, lv1, ttype, filter, t1, hardness, minlevel, maxlevel1, dwt_copy_scaling);
      vec_threshold_to(&wo, &y1o, lenh, lv1, ttype, filter, t1, hardness, minlevel, maxlevel1, dwt_copy_scaling);
      vec_transform(&y1e, lenh, lv1, ttype, filter, WO_BWD);
      vec_transform(&y1o, lenh, lv1, ttype, filter, WO_BWD);
      m1 = wo_interp_mse(xn, y1e.x, y1o.x, len);
    }
    iter++;
  }
  tc = m1 < m2 ? t1 : t2;
  if (trace) {
    trace->iters = iter;
    trace->t_final_raw = tc;
  }
  tc = tc / (sqrt(1. - log(2.) / log((double)len)));
  if (ttype == WO_DWT)
    threshold_dwt(w.x, NULL, len, tc, hardness, minlevel, maxlevel, levels, 0);
  else
    threshold_modwt(w.xmod, NULL, len, tc, hardness, minlevel, maxlevel, levels);
  vec_transform(&w, len, levels, ttype, filter, WO_BWD);
  vec_free(&y1e); vec_free(&y1o); vec_free(&y2e); vec_free(&y2o);
  vec_free(&we); vec_free(&wo);
  free(w.xmod);
  free(xn);
  return tc;
}

/* rfunctions.cu:71-100 */
int wo_smooth(double* x, int64_t len, int nlevels, int ttype, int filter,
              int threshtype, double* thresh, int hardness, int minlevel,
              int maxlevel, double tol) {
  int L = wo_filter_length(filter);
  int levels = wo_check_len_levels(len, nlevels, L);
  if (levels == 0) return 1;
  if (threshtype == 2) {
    *thresh = wo_cvt(x, len, levels, ttype, filter, hardness, tol, minlevel,
                     maxlevel, 0, NULL);
    return 0;
  }
  if (threshtype != 0 && threshtype != 1) return 2;
  double* xmod = NULL;
  if (ttype == WO_MODWT) {
    xmod = (double*)calloc((size_t)(2 * len * levels), sizeof(double));
    wo_modwt(x, xmod, len, WO_FWD, levels, filter);
  } else {
    wo_dwt(x, len, WO_FWD, levels, filter);
  }
  if (threshtype == 1) *thresh = wo_univ_thresh(x, xmod, len, levels, ttype, 0, 0);
  wo_threshold(x, xmod, len, levels, ttype, filter, *thresh, hardness, minlevel, maxlevel);
  if (ttype == WO_MODWT) wo_modwt(x, xmod, len, WO_BWD, levels, filter);
  else wo_dwt(x, len, WO_BWD, levels, filter);
  free(xmod);
  return 0;
}

void wo_count_kept(const double* x, const double* xmod, int64_t len,
                   int nlevels, int ttype, double t, int minlevel,
                   int maxlevel, int64_t* kept, int64_t* zeroed) {
  int64_t k = 0, z = 0;
  for (int l = minlevel; l <= maxlevel && l < nlevels; l++) {
    if (ttype == WO_DWT) {
      int64_t skip = (int64_t)1 << l;
      for (int64_t i = skip; i < len; i += 2 * skip) {
        if (fabs(x[i]) < t) z++; else k++;
      }
    } else {
      const double* d = xmod + (int64_t)(2 * l + 1) * len;
      for (int64_t i = 0; i < len; i++) {
        if (fabs(d[i]) < t) z++; else k++;
      }
    }
  }
  *kept = k;
  *zeroed = z;
}
