/*
 * measure_ia_gb300 -- C ABI of the GB300 (sm_103a) periodic-box pair counter.
 *
 * One call, mia_measure(), does what MeasureIA's box backends do for one
 * dataset: neighbour search, per-pair binning of DD, S+D and SxD (with the
 * jackknife parts), analytic RR, jackknife realisations, Pi integration or
 * Legendre multipoles, and the jackknife mean/std/covariance.  Inputs and
 * outputs are device pointers; scratch memory is a caller-provided device
 * buffer of mia_workspace_size() bytes.  The library allocates no memory.
 *
 * Reference interfaces replaced (MarloesvL/measure_IA, src/measureia/):
 *   mia_measure, kind MIA_KIND_W
 *     MeasureWBoxJackknife._measure_xi_rp_pi_box_jk_multiprocessing
 *       (measure_w_box_jk.py:648-857), ..._jk_tree (:293-541),
 *       ..._jk_brute (:69-291);
 *     MeasureWBox._measure_xi_rp_pi_box_multiprocessing
 *       (measure_w_box.py:493-656), ..._tree (:233-410), ..._brute (:65-231);
 *     then MeasureIABase._measure_w_g_i (measure_IA_base.py:515-575) and
 *       ._combine_jackknife_information (measure_IA_base.py:454-513).
 *   mia_measure, kind MIA_KIND_MULTIPOLES
 *     MeasureMBoxJackknife._measure_xi_r_mur_box_jk_multiprocessing
 *       (measure_m_box_jk.py:684-898), ..._jk_tree (:306-568),
 *       ..._jk_brute (:72-304);
 *     MeasureMultipolesBox._measure_xi_r_mur_box_multiprocessing
 *       (measure_m_box.py:719-890), ..._tree (:433-627), ..._brute (:255-431);
 *     then MeasureIABase._measure_multipoles (measure_IA_base.py:577-668)
 *       and ._combine_jackknife_information.
 *   mia_workspace_size / mia_output_layout: sizing helpers with no
 *     reference counterpart (the reference allocates numpy arrays inside
 *     each backend, e.g. measure_w_box_jk.py:749-759).
 *
 * Every function returns MIA_OK (0) or a nonzero MIA_ERR_* code; the
 * message of the last failure on a context is in mia_last_error().
 * A context is not re-entrant: use one context per host thread / stream.
 */
#ifndef MEASURE_IA_GB300_H
#define MEASURE_IA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define MIA_API __attribute__((visibility("default")))
#else
#define MIA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define MIA_OK 0
#define MIA_ERR_ARG 1        /* invalid argument (maps to ValueError)            */
#define MIA_ERR_CUDA 2       /* CUDA runtime error                               */
#define MIA_ERR_RANGE 3      /* coordinate outside [0, L) or not finite          */
#define MIA_ERR_OVERFLOW 4   /* edge re-test queue overflow in the mixed form    */
#define MIA_ERR_WORKSPACE 5  /* workspace missing, misaligned or too small       */

enum { MIA_KIND_W = 0, MIA_KIND_MULTIPOLES = 1 };
/* neighbour membership: TREE = the KD-tree backends (r_min < d <= r_max),
   BRUTE = temp_file_path=False (every pair inside the bin range). */
enum { MIA_TREE = 0, MIA_BRUTE = 1 };
enum { MIA_FP64 = 0, MIA_MIXED = 1 };
enum { MIA_DISTORTION = 0, MIA_ELLIPTICITY = 1 };

#define MIA_MAX_BINS_R 64
#define MIA_MAX_BINS_P 128
#define MIA_MAX_BREAKS 96

/* A catalogue as MeasureIABox.data holds it after masking: device pointers
   to float64 arrays in C order (measure_IA_base.py:81-95). */
typedef struct {
  const double* position;        /* (n_pos, 3)   'Position'                      */
  const double* weight;          /* (n_pos)      'weight'                        */
  const double* position_shape;  /* (n_shape, 3) 'Position_shape_sample'         */
  const double* axis_direction;  /* (n_shape, 2) 'Axis_Direction' (normalised here) */
  const double* q;               /* (n_shape)    'q'                             */
  const double* weight_shape;    /* (n_shape)    'weight_shape_sample'           */
  int64_t n_pos;
  int64_t n_shape;
} mia_catalog;

/* Measurement settings.  Host pointers.  The breakpoint tables encode the
   reference's exact bin assignment (see measure_ia_gb300/binning.py): for
   q = d^2 (r_p^2 for w, r^2 for multipoles) the bin is
   q_bin[#{k : q >= q_break[k]}] (-1 = not binned); likewise p_bin for the
   line-of-sight separation Pi (w) or mu_r = Pi / r (multipoles). */
typedef struct {
  int kind;            /* MIA_KIND_*                                       */
  int membership;      /* MIA_TREE | MIA_BRUTE                             */
  int precision;       /* MIA_FP64 | MIA_MIXED                             */
  int los;             /* line-of-sight axis 0, 1 or 2 ('LOS')             */
  int l_subboxes;      /* jackknife sub-boxes per side; 0 = no jackknife   */
  int ellipticity;     /* MIA_DISTORTION | MIA_ELLIPTICITY                 */
  int want_variance;   /* accumulate the sum of squared S+D terms          */
  int n_r;             /* num_bins_r                                       */
  int n_p;             /* num_bins_pi (Pi bins or mu_r bins)               */
  int n_qbreak;
  int n_pbreak;
  int shapes_per_unit; /* 0 = automatic (at most 256)                      */
  int cell_refine;     /* position cells per shape cell side in the projected
                          plane (and along the line of sight unless
                          cell_refine_los is set); 0 = automatic             */
  double boxsize;      /* L                                                */
  double volume;       /* L**3 as the reference forms it                   */
  double r_min, r_max; /* separation_limits                                */
  double rp_cut;       /* multipoles: pairs need r_p > rp_cut              */
  double cell_size;    /* target cell side in the projected plane (and along
                          the line of sight unless cell_size_los is set);
                          0 = automatic                                     */
  const double* r_edges;   /* n_r + 1 : r_bins                             */
  const double* p_edges;   /* n_p + 1 : pi_bins or mu_r_bins               */
  const double* q_break;   /* n_qbreak ascending                           */
  const int* q_bin;        /* n_qbreak + 1                                 */
  const double* p_break;   /* n_pbreak ascending                           */
  const int* p_bin;        /* n_pbreak + 1                                 */
  /* Launch geometry along the line of sight.  Cells that are narrow in the
     projected plane and long along the line of sight keep fewer out-of-range
     candidates per binned pair at the same shapes per cell.  Results do not
     depend on these (nor on cell_size, cell_refine, shapes_per_unit). */
  double cell_size_los;    /* target cell side along the LOS; 0 = cell_size */
  int cell_refine_los;     /* position cells per shape cell along the LOS;
                              0 = cell_refine                               */
} mia_config;

/* Offsets (in doubles) of every product inside the output buffer.
   nb = n_r * n_p; J = number of jackknife regions (0 without jackknife).
   Histograms hold raw sums (no 1/(2R) factor): [0] = all pairs,
   [1 + i] = pairs with the shape or the position in region i. */
typedef struct {
  int64_t total;
  int64_t dd;          /* (1+J) * nb                                         */
  int64_t splus;       /* (1+J) * nb   sum w_p w_s e_+                        */
  int64_t scross;      /* nb           sum w_p w_s e_x                        */
  int64_t variance;    /* nb           sum (w_p w_s e_+ / 2R)^2               */
  int64_t npos_jk;     /* J   positions outside region i                    */
  int64_t nshape_jk;   /* J   shapes outside region i                       */
  int64_t R;           /* 1   responsivity                                  */
  int64_t R_jk;        /* J                                                 */
  int64_t rr;          /* nb  analytic RR                                    */
  int64_t rr_jk;       /* J * nb                                            */
  int64_t xi_gp, xi_gx, xi_gg, splusd, scrossd, sigmasq; /* nb each         */
  int64_t xi_gp_jk, splusd_jk, xi_gg_jk, dd_jk;          /* J * nb each     */
  int64_t proj_gp, proj_gg;          /* n_r : w or multipole, full sample    */
  int64_t proj_gp_jk, proj_gg_jk;    /* J * n_r                              */
  int64_t mean_gp, std_gp, cov_gp;   /* n_r, n_r, n_r * n_r                  */
  int64_t mean_gg, std_gg, cov_gg;
  int64_t stats;       /* 8: n_pos, n_shape, binned pairs, edge pairs
                          re-tested, work units, cells, pair launches, 0    */
} mia_layout;

typedef struct {
  double* out;                  /* layout.total doubles (device)           */
  unsigned long long* npairs;   /* (1+J) * nb integer pair counts (device) */
} mia_result;

/* Context on one device (the device must be current on the calling thread). */
typedef struct mia_context mia_context;

MIA_API int mia_create(int device, mia_context** ctx);
MIA_API int mia_destroy(mia_context* ctx);
MIA_API const char* mia_last_error(const mia_context* ctx);
MIA_API int mia_version(void);

/* Bytes of device scratch mia_measure needs for this configuration. */
MIA_API int mia_workspace_size(const mia_config* cfg, int64_t n_pos, int64_t n_shape, size_t* bytes);

/* Output offsets for this configuration. */
MIA_API int mia_output_layout(const mia_config* cfg, mia_layout* layout);

/* The whole measurement, enqueued on `stream` (a cudaStream_t, 0 = legacy
   default stream).  Returns after the results are complete on the device;
   the catalogue, workspace and result buffers must stay valid until then. */
MIA_API int mia_measure(mia_context* ctx, const mia_config* cfg, const mia_catalog* cat, void* workspace,
                size_t workspace_bytes, const mia_result* res, void* stream);

/* ---- batches: many catalogues, one binning, one persistent pair kernel ----
   Many catalogues measured with the same configuration (e.g. mass or colour
   subsamples of several snapshots) share one launch of the pair kernel: a
   global work counter walks the work units of every catalogue, largest
   workloads balance with the small ones.  Replaces repeated calls of the
   backends above, one catalogue at a time (the reference's Pool.map covers
   one catalogue, measure_w_box_jk.py:765-780).
   mia_batch_prepare uploads tables and descriptors (synchronous, not
   capturable); mia_batch_enqueue only enqueues memsets and kernels, so it can
   be captured in a CUDA graph and replayed; mia_batch_status reads the
   catalogues' error flags after the work completes.  results[i] receives
   catalogue i's products in the layout of mia_output_layout. */
MIA_API int mia_batch_workspace_size(const mia_config* cfg, int n, const int64_t* n_pos, const int64_t* n_shape,
                                     size_t* bytes);
MIA_API int mia_batch_prepare(mia_context* ctx, const mia_config* cfg, int n, const mia_catalog* cats,
                              void* workspace, size_t workspace_bytes, const mia_result* results, void* stream);
MIA_API int mia_batch_enqueue(mia_context* ctx, const mia_config* cfg, int n, const mia_catalog* cats,
                              void* workspace, size_t workspace_bytes, const mia_result* results, void* stream);
MIA_API int mia_batch_status(mia_context* ctx, int n, void* workspace, void* stream);
MIA_API int mia_measure_batch(mia_context* ctx, const mia_config* cfg, int n, const mia_catalog* cats,
                              void* workspace, size_t workspace_bytes, const mia_result* results, void* stream);


/* Jackknife covariance of two datasets (or of one with itself: pass the same
   pointer twice), on device, from their realisations: real_a and real_b hold
   n_real rows of n_bins doubles (row starts stride_a / stride_b doubles
   apart; e.g. the proj_gp_jk block of two mia_measure outputs).  Writes
   cov (n_bins x n_bins, row-major, cov[j][i] pairs a's bin j with b's bin i)
   and std (n_bins) as the reference forms them: f = (n_real - 1) / n_real,
   cov = f * sum_r (a_r - mean_a)(b_r - mean_b)^T, std = sqrt(f * sum_r
   (a_r - mean_a)(b_r - mean_b)) elementwise (NaN where that is negative).
   All pointers are device memory; enqueued on `stream`.  Replaces
   MeasureJackknife.measure_covariance_multiple_datasets
   (measure_jackknife.py:485-571) without the HDF5 round trip. */
MIA_API int mia_jackknife_cross_cov(mia_context* ctx, int n_real, int n_bins, const double* real_a, int64_t stride_a,
                                    const double* real_b, int64_t stride_b, double* cov, double* std, void* stream);

/* Opt-in timing of the pair kernel (the dominant stage), for profiling: with
   n_slots > 0 every later mia_measure / mia_batch_enqueue on this context
   records a CUDA event pair around its pair-kernel launch, on the caller's
   stream, into a ring of n_slots entries; n_slots = 0 switches it off.
   mia_profile_read waits for and returns the durations (ms) of the last
   min(n, recorded, n_slots) launches, oldest first, in *n_out.  No counterpart
   in the reference (its Pool has no device stage to time). */
MIA_API int mia_profile_pairs(mia_context* ctx, int n_slots);
MIA_API int mia_profile_read(mia_context* ctx, float* ms, int n, int* n_out);

/* Size of the library's own device scratch used by mia_measure_static. */
#define MIA_STATIC_SCRATCH_BYTES (64ull * 1024ull * 1024ull)

/* mia_measure without a workspace argument, for callers that cannot allocate
   device memory: code running under a host application or plugin framework
   that owns the whole GPU memory budget and hands out no scratch, or a loop
   that must not call cudaMalloc because it synchronises the device.  The
   scratch is a 64 MiB array in the library's device module, held on every
   GPU that loads the library until the process exits.  Measurements whose
   scratch need (mia_workspace_size) exceeds MIA_STATIC_SCRATCH_BYTES are
   rejected with MIA_ERR_WORKSPACE; invalid arguments get mia_measure's
   errors and messages.  Each call looks up the array's device address
   (cudaGetSymbolAddress) with the context's device current; a device's
   first call also loads the library's module there, so make that first call
   before any stream capture (after a cudaDeviceReset the next call finds the
   array's new address).  All calls share the one array, so calls that
   overlap on the GPU (other streams, other host threads) race; every call
   clears what must start at zero.  Inputs and outputs are still
   caller-provided device buffers.  No counterpart in the reference. */
MIA_API int mia_measure_static(mia_context* ctx, const mia_config* cfg, const mia_catalog* cat,
                               const mia_result* res, void* stream);

/* ---- lightcone pair counts -------------------------------------------------

   One brute-force lightcone counter of MeasureIALightcone, for one pair of
   samples ("positions" = the outer loop of the reference, "shapes" = the
   inner one), and all of its jackknife realisations in the same pass:

     with_shapes = 1, w : _measure_xi_rp_pi_lightcone_brute  (measure_w_lightcone.py:45-214)
     with_shapes = 0, w : _count_pairs_xi_rp_pi_lightcone_brute (measure_w_lightcone.py:216-343)
     with_shapes = 1, m : _measure_xi_r_mur_lightcone_brute  (measure_m_lightcone.py:45-219)
     with_shapes = 0, m : _count_pairs_xi_r_mur_lightcone_brute (measure_m_lightcone.py:221-363)

   and the per-patch re-counts of the pooled jackknife driver
   (measure_jackknife.py:265-484), which drop every pair with either member in
   the patch.  Per pair the separations are the reference's flat-sky ones in
   the position's frame, computed in FP64 in the reference's operation order:
     dx = ((ra_s - ra_p) / 180 * pi) * chi_p * cos_dec_p,  dy = ((dec_s - dec_p) / 180 * pi) * chi_p,
     Pi = chi_s - chi_p,  w: q = (h_extra dx)^2 + (h_extra dy)^2,
     m: q = (dx^2 + dy^2) + Pi^2, r_p^2 = (h_extra dx)^2 + (h_extra dy)^2, mu = Pi / sqrt(q).
   Bins come from breakpoint tables: q_bin over q (w: r_p^2, m: r^2) and p_bin
   over Pi (w) or mu (m), each -1 for "not binned" and -2 for an index past the
   last bin (where the reference's np.add.at raises IndexError; such pairs set
   MIA_LC_INDEX_ERROR in *status and are not counted).  S+D / SxD use
   e+ = -e cos 2(phi_a - phi_s), ex = -e sin 2(phi_a - phi_s) from the shape's
   cos 2 phi_a, sin 2 phi_a and the separation direction (0 where r_p = 0).

   Outputs (device): out[q][k][bin] for q = DD, S+D, SxD (S+D and SxD only
   with with_shapes) and k = 0 (all pairs) or 1 + i (pairs with neither member
   in patch i), bin = r * n_p + p; counts[k][bin] = pair counts (int64).  Sums
   are raw: the reference's "DD == 0 -> 1" and the estimators are host work. */

#define MIA_LC_INDEX_ERROR 1u
#define MIA_LC_BAD_PATCH 2u       /* a position label outside 0..n_patch-1 (position skipped),
                                     or a shape label >= n_patch (treated as -1) */

typedef struct {
  int kind;                 /* MIA_KIND_W or MIA_KIND_MULTIPOLES */
  int with_shapes;          /* 1: DD, S+D, SxD; 0: DD only */
  int n_r, n_p;
  int n_patch;              /* jackknife patches 0..n_patch-1; 0 = no realisations */
  int n_qbreak, n_pbreak;
  const double* q_break;    /* host arrays, as in mia_config */
  const int* q_bin;
  const double* p_break;
  const int* p_bin;
  double h_extra;           /* factor on the projected separation (h with over_h, else 1) */
  double rp_cut;            /* multipoles: a pair needs r_p > rp_cut */
  double r_lim;             /* r_bins[-1]: no pair at or beyond it is binned */
  double pi_lo, pi_hi;      /* w: binned Pi range [pi_lo, pi_hi) */
  /* cell grid over the shapes (host-chosen; objects outside go to the edge cells) */
  double ra0, ra_cell, dec0, dec_cell, chi0, chi_cell;
  int n_ra, n_dec, n_chi;
  int unit_weights;         /* 1: every weight of both samples is exactly 1.0, so DD is the
                               pair count (the reference's sum of ones) and is not summed */
  int wide_sums;            /* sums are exact fixed-point integers; 0: a term keeps every bit
                               down to 2^-46 of the largest possible term (64-bit warp
                               partials), 1: down to 2^-88 (128-bit partials, more shared
                               memory); for weights spanning more than ~2^12 */
} mia_lc_config;

typedef struct {            /* device arrays of n entries */
  int64_t n;
  const double *ra, *dec, *chi, *w;
  const double* cos_dec;    /* positions: cos(dec / 180 * pi) as numpy forms it */
  const double *e, *c2a, *s2a;  /* shapes with with_shapes: |e|, cos 2 phi_a, sin 2 phi_a */
  const int32_t* patch;     /* 0..n_patch-1, or -1 (in no realisation's patch); NULL when n_patch = 0 */
} mia_lc_sample;

MIA_API int mia_lc_workspace_size(const mia_lc_config* cfg, int64_t n_pos, int64_t n_shape, size_t* bytes);
MIA_API int mia_lc_count(mia_context* ctx, const mia_lc_config* cfg, const mia_lc_sample* pos,
                         const mia_lc_sample* shape, void* workspace, size_t workspace_bytes, double* out,
                         int64_t* counts, uint32_t* status, void* stream);

#ifdef __cplusplus
}
#endif
#endif
