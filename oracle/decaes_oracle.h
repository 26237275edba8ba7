/*
 * decaes_oracle.h -- CPU oracle for the DECAES.jl v0.6.1 voxelwise T2 path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64 restatement of the
 * reference algorithm (T2mapSEcorr + T2partSEcorr and everything they call),
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker.  The GPU product never links, loads or calls it.
 *
 * Parity status: the reference is Julia and cannot run here, and it ships no
 * golden vectors.  Components are pinned against the known answers in the
 * reference's own test suite (test/optimization.jl, test/splines.jl,
 * test/nnls.jl, test/epg.jl); whole-pipeline parity against the Julia
 * reference is unpinned.  Deliberate deviations (all in branches the reference
 * marks as unreachable, or where its saved output depends on thread schedule)
 * are listed at each function.
 *
 * Arrays are column-major (Julia layout): image[v + V*e], dist[v + V*j].
 */
#ifndef DECAES_ORACLE_H
#define DECAES_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_REG_NONE = 0, ORC_REG_LCURVE = 1, ORC_REG_GCV = 2, ORC_REG_CHI2 = 3, ORC_REG_MDP = 4 };

/* Mirrors T2mapOptions{Float64} (src/types.jl:19-100); NaN = `nothing`. */
typedef struct {
    int nTE;
    double TE;
    int nT2;
    double T2Range[2];
    double T1;
    double Threshold;
    double MinRefAngle;
    int nRefAngles;
    int nRefAnglesMin;
    int Reg;
    double Chi2Factor;
    double NoiseLevel;
    double RefConAngle;
    double SetFlipAngle;
    int legacy;          /* legacy algorithms: spline surrogate, chi2 doubling search */
} orc_t2map_opts;

/* Output buffers of T2mapSEcorr (src/T2mapSEcorr.jl:2-19); NULL = not saved.
 * Maps are V long, dist is V x nT2, decaycurve V x nTE. */
typedef struct {
    double *dist;
    double *gdn, *ggm, *gva, *fnr, *snr, *alpha;
    double *resnorm, *decaycurve, *mu, *chi2factor;
} orc_t2map_out;

/* Mirrors T2partOptions{Float64} (src/types.jl:139-172). */
typedef struct {
    int nT2;
    double T2Range[2];
    double SPWin[2];
    double MPWin[2];
    double Sigmoid; /* NaN = nothing */
} orc_t2part_opts;

typedef struct {
    double *sfr, *sgm, *mfr, *mgm;
} orc_t2part_out;

/* Stage indices of the FP64 operation counters. */
enum {
    ORC_ST_ENSEMBLE = 0, /* EPG angle-ensemble basis + derivative */
    ORC_ST_SEARCH_NNLS,  /* unregularized NNLS solves of the flip-angle search */
    ORC_ST_SEARCH_OTHER, /* gradients, spline surrogate */
    ORC_ST_BASIS,        /* per-voxel EPG basis at the optimal angle */
    ORC_ST_REG_NNLS,     /* NNLS solves inside the regularizer */
    ORC_ST_REG_OTHER,    /* root finding, curvature, GCV dof */
    ORC_ST_SVD,          /* GCV singular values */
    ORC_ST_SAVE,         /* save_results! epilogue */
    ORC_ST_T2PART,
    ORC_NSTAGES
};

/* ---- whole-path entry points ---- */
int orc_t2map(const orc_t2map_opts *o, const double *image, long V, const double *b1map,
              orc_t2map_out *out, int nthreads, double *flops /* ORC_NSTAGES or NULL */);
int orc_t2part(const orc_t2part_opts *o, const double *dist, long V, orc_t2part_out *out, int nthreads);

/* ---- synthetic benchmark image (the same bytes as decaes_mock_image) ---- */
typedef struct {
    int nTE;
    double TE;
    double T1;
    double FlipAngleRange[2];   /* degrees, uniform */
    double MyelinT2Range[2];    /* seconds */
    double MyelinFracRange[2];
    double IET2Range[2];
    double CSFT2Range[2];
    double CSFFracRange[2];
    double AmplitudeRange[2];
    double SNRRange[2];         /* linear SNR; noise sigma = amplitude / SNR */
    double BackgroundFraction;  /* voxels with zero amplitude (noise only) */
    double BackgroundSigma;
} orc_mock_opts;
/* image[v + V*e] for voxels 0..V-1 (a leading slab of a larger volume is the
 * same bytes as that volume's first V voxels); f32 != 0 writes floats. */
int orc_mock_image(const orc_mock_opts *o, uint64_t seed, long V, void *image, int f32, int nthreads);

/* ---- grids ---- */
void orc_linrange(double a, double b, int len, double *out);
void orc_logrange(double a, double b, int len, double *out);
double orc_sind(double x);
double orc_erfinv(double x);

/* ---- EPG ---- */
void orc_epg_decay_curve(int ETL, double alpha, double TE, double T2, double T1, double beta, double *dc);
void orc_epg_decay_curve_dual(int ETL, double alpha, double TE, double T2, double T1, double beta,
                              double *dc, double *ddc);
void orc_epg_decay_curve_basic(int ETL, double alpha, double TE, double T2, double T1, double beta, double *dc);

/* ---- NNLS and regularizers on an explicit (A, b) ---- */
int orc_nnls(const double *A, int m, int n, const double *b, double *x, double *rnorm, int *nsetp, int *mode);
int orc_lsqnonneg(const double *A, int m, int n, const double *b, double *x, double *rnorm, int *nsetp);
int orc_lsqnonneg_tikh(const double *A, int m, int n, const double *b, double mu, double *x,
                       double *loss, double *seminorm_sq, double *resnorm_sq, int *nsetp);
int orc_lsqnonneg_chi2(const double *A, int m, int n, const double *b, double chi2_target,
                       double *x, double *mu, double *chi2);
int orc_lsqnonneg_mdp(const double *A, int m, int n, const double *b, double delta,
                      double *x, double *mu, double *chi2);
int orc_lsqnonneg_lcurve(const double *A, int m, int n, const double *b, double *x, double *mu, double *chi2);
int orc_lsqnonneg_gcv(const double *A, int m, int n, const double *b, double *x, double *mu, double *chi2);
int orc_svdvals(const double *A, int m, int n, double *s);
int orc_lsqnonneg_chi2_legacy(const double *A, int m, int n, const double *b, double chi2_target,
                              double *x, double *mu, double *chi2);

/* legacy spline machinery (FITPACK restatement, Julia float ranges) */
int orc_jl_colon(double start, double step, double stop, double *out, long maxlen, long *len);
int orc_fitpack_curfit0(const double *x, const double *y, int m, int k, double *t, double *c);
int orc_fitpack_splev(const double *t, int n, const double *c, int k, const double *x, int npts, double *y);
int orc_spline_opt_legacy(const double *X, const double *Y, int npts, double *x, double *y);
int orc_spline_root_legacy(const double *X, const double *Y, int npts, double value, double *x);

/* ---- scalar optimizers with a callback ---- */
typedef double (*orc_fn)(double x, void *ctx);
typedef void (*orc_fn2)(double x, double *P, void *ctx);
void orc_brent_root(orc_fn f, void *ctx, double a, double b, double xatol, double xrtol, double ftol,
                    int maxiters, double *x, double *fx);
void orc_bisect_root(orc_fn f, void *ctx, double a, double b, double xatol, double xrtol, double ftol,
                     int maxiters, double *x, double *fx);
void orc_brent_minimize(orc_fn f, void *ctx, double a, double b, double xatol, double xrtol, int maxiters,
                        double *x, double *fx);
double orc_lcurve_corner(orc_fn2 f, void *ctx, double xlow, double xhigh, double xtol, double Ptol, double Ctol);

/* ---- flip-angle surrogate search pieces (1-based grid indices, as in the reference) ---- */
void orc_cubic_hermite_minimize(double a, double b, double u0, double u1, double m0, double m1,
                                double *x, double *u);
int orc_minimal_bounding_box(int K, const double *grid, const unsigned char *seen, double x, int *lo, int *hi);

#ifdef __cplusplus
}
#endif
#endif
