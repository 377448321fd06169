/*
 * wavoracle: CPU restatement of the wavecuda reference's FP64 CPU path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU baseline.  The product library
 * (libwavecuda_gb300.so) never links, loads or calls it.
 *
 * Parity pinning: every function here is checked against the reference's own
 * CPU sources compiled from the reference tree (oracle/_ref/libwavref.so) on
 * golden inputs; the resulting fixtures live in tests/golden/.  C6 and LA8
 * MODWT have no reference implementation; their restatement is the generic
 * a-trous form of daub4.cpp:561-589 with the C6/LA8 taps, pinned through its
 * Haar/D4 instances and through perfect reconstruction.
 *
 * Codes follow wvtheads.h:14-38: FWD 1 / BWD 0; HAAR 1, DAUB4 2, C6 3, LA8 4;
 * DWT 0, MODWT (time ordered) 1; HARD 0 / SOFT 1.  Levels are 0-based.
 */
#ifndef WAVORACLE_H
#define WAVORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Filter length of a filter code (wavutils.cpp:784-806); 0 if unknown. */
int wo_filter_length(int filter);

/* check_len_levels (wavutils.cpp:48-64): 0 on error, else the level count. */
int wo_check_len_levels(int64_t len, int nlevels, int filterlen);

/* Threads of the per-level transform loops (n <= 0: every core).  Results do
 * not depend on it. */
void wo_set_threads(int n);
int wo_get_threads(void);

/* DWT, interleaved in place (haar.cpp:9-30). */
int wo_dwt(double* x, int64_t len, int sense, int nlevels, int filter);

/* Time-ordered MODWT (haar.cpp:561-685, daub4.cpp:495-589): xmod holds
 * [s_1 | d_1 | s_2 | d_2 | ...], 2*len*nlevels doubles.  FWD reads x and
 * writes xmod; BWD reads s_J and d_1..d_J from xmod and writes x (the
 * intermediate s blocks are used as scratch, as in the reference). */
int wo_modwt(double* x, double* xmod, int64_t len, int sense, int nlevels,
             int filter);

/* Packet-ordered MODWT (code 2; haar.cpp:305-398, daub4.cpp:392-484), any
 * filter.  FWD: x -> xmod (2*len*J values, packet order).  BWD: xmod -> x. */
int wo_modwt_po(double* x, double* xmod, int64_t len, int sense, int nlevels, int filter);

/* thresh_coef (thresh.cpp:142-157). */
double wo_thresh_coef(double coef, double thresh, int hardness);

/* threshold(wst*,NULL,...) with level limits (thresh.cpp:113-140), in place.
 * Returns 0 when the level limits were accepted and the data thresholded. */
int wo_threshold(double* x, double* xmod, int64_t len, int nlevels, int ttype,
                 int filter, double thresh, int hardness, int minlevel,
                 int maxlevel);

/* median / mad (utils.cpp:166-203). x is not modified. */
double wo_median(const double* x, int64_t len);
double wo_mad(const double* x, int64_t len);

/* univ_thresh (thresh.cpp:170-201) on a transformed vector. */
double wo_univ_thresh(const double* x, const double* xmod, int64_t len,
                      int nlevels, int ttype, int minlevel, int maxlevel);

/* interp_mse (thresh.cpp:344-385). */
double wo_interp_mse(const double* xn, const double* ye, const double* yo,
                     int64_t len);

/* Golden-section trace of one CVT run. */
typedef struct {
  int iters;            /* loop iterations executed */
  double t1[64], t2[64];/* t1/t2 at each comparison (index = iteration) */
  double m1[64], m2[64];/* losses compared at each iteration */
  int took_m2[64];      /* 1 where m2 < m1 */
  double t_final_raw;   /* m1<m2 ? t1 : t2 before the rescale */
  double t_univ;        /* bracket upper end */
} wo_cv_trace;

/* CVT (thresh.cpp:203-342).  x (len doubles) is replaced by the smoothed
 * signal; returns the chosen threshold.  trace may be NULL.
 * dwt_copy_scaling = 0 reproduces the reference's threshold_dwt, which leaves
 * the coarse scaling slots k*2^(J-1), k>0, of the half-length work vectors
 * unwritten (they keep the previous inverse transform's values; zero at the
 * start); 1 copies them as a full threshold would. */
double wo_cvt(double* x, int64_t len, int nlevels, int ttype, int filter,
              int hardness, double tol, int minlevel, int maxlevel,
              int dwt_copy_scaling, wo_cv_trace* trace);

/* RcpuSmooth (rfunctions.cu:71-100). threshtype 0 manual, 1 univ, 2 cv. */
int wo_smooth(double* x, int64_t len, int nlevels, int ttype, int filter,
              int threshtype, double* thresh, int hardness, int minlevel,
              int maxlevel, double tol);

/* Kept/zeroed counts of the detail coefficients in [minlevel, maxlevel]
 * under threshold t (|c| < t is zeroed, thresh.cpp:143). */
void wo_count_kept(const double* x, const double* xmod, int64_t len,
                   int nlevels, int ttype, double t, int minlevel,
                   int maxlevel, int64_t* kept, int64_t* zeroed);

#ifdef __cplusplus
}
#endif
#endif
