// Internal definitions shared by the measure_ia_gb300 CUDA translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/measure_ia_gb300.h"

namespace mia {

// --------------------------------------------------------------------------
// Sizes
// --------------------------------------------------------------------------
constexpr int kThreads = 256;            // pair-kernel block size
constexpr int kLutBits = 11;             // 2048-bucket logarithmic lookup table (32 octaves)
constexpr int kLut = 1 << kLutBits;
constexpr int kLutMantBits = 6;          // 64 buckets per octave of q
constexpr int kScanTile = 2048;
constexpr int kLutReject = 0x7FFF;       // lutw: clean bucket whose q is not binned
constexpr int kHistShort = 1920;         // u32 words per replicated histogram array, short pair path
constexpr int kHistShortVar = 1536;      // the same with variance terms (five arrays)

// status word bits
constexpr unsigned kStatusRange = 1u;      // input coordinate outside [0, L) or NaN
constexpr unsigned kStatusOverflow = 2u;   // edge queue overflow
constexpr unsigned kStatusNoSlot = 4u;     // (informational) global-atomic fallback used

// --------------------------------------------------------------------------
// Device-visible status block (first bytes of the workspace)
// --------------------------------------------------------------------------
struct Status {
  unsigned flags;
  unsigned pad;
  unsigned long long edge_count;       // pairs queued for the FP64 re-test
  unsigned long long wu_next;          // persistent-kernel work counter
  unsigned long long n_wu;             // number of work units
  unsigned long long binned;           // binned pairs (all regions, once each)
  unsigned long long bad_index;        // first offending input index (range check)
  unsigned long long maxw_bits;        // max |w_p| (bit pattern; non-negative doubles order as integers)
  unsigned long long maxws_bits;       // max(|w_s|, |w_s e|)
};

// Exact bin tables, built on the host from the reference's formulas.
struct Tables {
  // q = d^2 breakpoints (FP64) and their keys; bins of the intervals between them
  double q_break[MIA_MAX_BREAKS];
  long long q_key[MIA_MAX_BREAKS];     // bit pattern of q_break (q >= 0, so integer order = value order)
  int q_bin[MIA_MAX_BREAKS + 1];
  // FP32 guard band around each q breakpoint: q < q_lo32 -> surely below, q >= q_hi32 -> surely above
  float q_lo32[MIA_MAX_BREAKS];
  float q_hi32[MIA_MAX_BREAKS];
  // Pi or mu breakpoints, keys in signed-order form
  double p_break[MIA_MAX_BREAKS];
  long long p_key[MIA_MAX_BREAKS];
  int p_bin[MIA_MAX_BREAKS + 1];
  // lookup tables: bucket -> bin + 1, or first breakpoint index | 0x8000
  // (the bucket touches a guard band)
  unsigned short lut32[kLut];
  // the same buckets for the short pair path: a clean bucket holds ib * n_p
  // (kLutReject when not binned), a bucket touching a guard band its qdirty
  // entry | 0x8000.  That path only looks up
  // q <= q_cut, which lies below the last bucket, and an index below the
  // table wraps (unsigned) to the last bucket: it holds the bin under the
  // first breakpoint
  unsigned short lutw[kLut];
  // short path, buckets touching a guard band (lutw entry 0x8000 | index):
  // (band_lo, band_hi, code below, code above) -- the union of the guard
  // bands that meet the bucket; a q below it takes the code below (ib * n_p
  // or kLutReject, as int bits), above it the code above, inside it is an
  // edge
  float4 qdirty[MIA_MAX_BREAKS];
  // bin edges (r_bins; pi_bins or mu_r_bins)
  double r_edges[MIA_MAX_BINS_R + 1];
  double p_edges[MIA_MAX_BINS_P + 1];
};

// --------------------------------------------------------------------------
// Plan: geometry of the cell grid and the workspace carve-up
// --------------------------------------------------------------------------
struct Plan {
  // geometry, in cell-dimension order d0, d1 (projected plane), d2 (line of sight)
  int axis[3];          // original axis of d0, d1, d2
  int n[3];             // shape cells per dimension (coarse grid)
  double s[3];          // shape cell side
  int R[3];             // neighbour reach in coarse cells
  int m[3];             // position cells per shape cell along each dimension
  int nf[3];            // position cells per dimension (fine grid, nf = m * n)
  double sf[3];         // position cell side
  int Rf[3];            // neighbour reach in position cells
  int full[3];          // the reach covers the box: every position cell is visited, per-pair wrap
  long long n_fcells;
  int n_sub;            // jackknife sub-boxes per side (1 when no jackknife)
  int J;                // number of jackknife regions (0 when none)
  long long n_cells;
  double range_proj;    // largest binned projected separation (or 3-D for multipoles)
  double range_los;     // largest binned |Pi| (w) or r (multipoles)
  int shapes_per_unit;
  long long n_wu_max;
  long long edge_capacity;
  int nb;
  // workspace offsets in bytes
  size_t off_status, off_tables;
  size_t off_pcount, off_pstart, off_pcur, off_scount, off_sstart, off_scur_lo, off_scur_hi;
  size_t off_wucount, off_wustart, off_tiles;
  size_t off_pcell, off_plab, off_scell, off_slab;
  size_t off_p64, off_plab_s, off_p32;
  size_t off_s64, off_slab_s, off_s32;
  size_t off_wu;
  size_t off_reg;
  size_t off_edges;
  size_t off_acc;
  int acc_words;        // 64-bit words per fixed-point sum: 1 (mixed form) or 2 (FP64 form)
  size_t total;
};

// Work unit: a run of shapes of one cell with one jackknife label.
struct WorkUnit {
  int cell;
  int begin;   // first shape (sorted order)
  int count;
  int label;   // jackknife region of every shape in the unit
};

// Region accumulators (per jackknife region, plus the totals at index J).
struct RegionStats {
  unsigned long long* npos;     // J + 1
  unsigned long long* nshape;   // J + 1
  double* s1;                   // J + 1 : sum w_s (1 - e^2/2)
  double* s2;                   // J + 1 : sum w_s
  long long* r1;                // J + 1 : s1 and s2 as exact fixed-point sums (scale
  long long* r2;                //         region_scale), converted into s1, s2
};

// Fixed-point scale of the responsivity sums: 2^S with n * max|w_s| * 2^S <=
// 2^62, so no total of n shapes can overflow and a term keeps ~62 - log2(n)
// bits.  Integer sums make R independent of the order of the adds.
__device__ inline double region_scale(unsigned long long maxws_bits, long long n_shape) {
  double m = __longlong_as_double((long long)maxws_bits) * (double)(n_shape > 0 ? n_shape : 1);
  if (!(m > 0.0) || !(m < 1e300)) m = 1.0;
  int e = ilogb(4611686018427387904.0 / m);  // 2^62
  e = e > 200 ? 200 : (e < -200 ? -200 : e);
  return ldexp(1.0, e);
}

// ---- exact 128-bit fixed-point sums (FP64 form) ------------------------------
//
// A term v enters a sum as the integer nearest v * 2^E (ties away from zero),
// a two's-complement 128-bit value in two 64-bit words (lo, hi).  E is chosen
// per dataset so that the largest possible term is at most 2^88: a term keeps
// every bit down to 2^-88 of the largest one, and a sum has room for 2^38
// terms of the largest size.  Adding the words is exact and commutative, so a
// sum does not depend on the order in which the pairs arrive; it is rounded
// to a double once, at the end.  Infinities and NaNs cannot be represented and
// are left to the caller (they go to the output doubles directly, so that a
// bin holding one reads inf or NaN as a plain sum would).
struct Fix128 {
  unsigned long long lo, hi;
};

// E with m * 2^E <= 2^88 (m > 0 finite), limited so that 2^-E is a normal double.
__device__ inline int fix128_exponent(double m) {
  if (!(m > 0.0) || !(m < 1e300)) m = 1.0;
  const int e = ilogb(309485009821345068724781056.0 / m);  // 2^88
  return e > 1000 ? 1000 : (e < -1000 ? -1000 : e);
}

// v * 2^E to the nearest integer, from v's bit fields (integer arithmetic
// only); false when v is not finite or |v| 2^E reaches 2^126.
__device__ __forceinline__ bool to_fix128(double v, int E, Fix128& f) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int be = (int)((bits >> 52) & 0x7ff);
  unsigned long long mant = bits & 0xFFFFFFFFFFFFFull;
  f.lo = 0;
  f.hi = 0;
  if (be == 0x7ff) return false;
  if (be) mant |= 1ull << 52;
  const int sh = (be ? be : 1) - 1075 + E;  // |v| 2^E = mant 2^sh
  if (sh >= 0) {
    if (sh > 126 - 53) return false;
    if (sh >= 64) {
      f.hi = mant << (sh - 64);
    } else {
      f.lo = mant << sh;
      f.hi = sh ? mant >> (64 - sh) : 0ull;
    }
  } else if (sh > -64) {
    const int s = -sh;
    f.lo = (mant + (1ull << (s - 1))) >> s;   // mant < 2^53: no overflow
  }
  if (bits >> 63) {
    f.lo = ~f.lo + 1ull;
    f.hi = ~f.hi + (f.lo == 0ull ? 1ull : 0ull);
  }
  return true;
}

// a[0..1] += f with 64-bit atomics: the carry out of the low word is read
// from the value the low-word add returned, so concurrent adds never lose one.
__device__ __forceinline__ void add_fix128(unsigned long long* a, const Fix128& f) {
  const unsigned long long old = atomicAdd(a, f.lo);
  const unsigned long long c = f.hi + (old + f.lo < old ? 1ull : 0ull);
  if (c) atomicAdd(a + 1, c);
}

// The sum (lo, hi) times inv (= 2^-E) as a double: the magnitude's two words
// are converted and added in round-to-nearest (deterministic; within 2 ulp).
__device__ __forceinline__ double fix128_value(unsigned long long lo, unsigned long long hi, double inv) {
  const bool neg = (long long)hi < 0;
  if (neg) {
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  double m = __dadd_rn(__dmul_rn(__ull2double_rn(hi), 18446744073709551616.0), __ull2double_rn(lo));
  m = __dmul_rn(m, inv);
  return neg ? -m : m;
}

// Fixed-point scales of one dataset (powers of two), from its largest weight
// product m = max|w_p| * max(|w_s|, |w_s e|) and responsivity R:
//   S+D, SxD : |term| * 2^S <= 2^30 -- signed terms, typically a few per cent
//              of the largest, so a work unit's partial of one (copy, bin)
//              random-walks inside 2^31; the rounding is far below the FP32
//              error of a term, which the cancelling bins of w_g+ need
//   w        : |term| * 2^S <= 2^24 -- a positive sum that only grows: it wraps
//              a 32-bit partial once per ~10^3 adds
//   var      : (|term| / 2R)^2 * 2^S <= 2^30 -- positive squares, but only the
//              brute layout with jackknife regions accumulates them, and there
//              each one is divided by RR^2: a one-pair bin of a small term at
//              small r needs the finer unit (2^22 left 5e-5 relative errors)
// The staged shape weights carry sc_dd (w_s) and sc_sp (w_s e), so a pair's
// terms come out scaled; c_vr maps a scaled S+D term to its variance term.
struct Scales {
  float sc_dd, sc_sp, c_vr;
  double inv_dd, inv_sp, inv_vr;
  double sd_dd, sd_sp, sd_vr;   // the scales as doubles (edge re-test)
  int e128, e128v;              // FP64 form: 128-bit fixed-point exponents (w, S+D, SxD; variance)
  double inv128, inv128v;       // 2^-e128, 2^-e128v
};

__device__ inline Scales dataset_scales(const Status* st, double twoR) {
  double m = __longlong_as_double((long long)st->maxw_bits) * __longlong_as_double((long long)st->maxws_bits);
  if (!(m > 0.0) || !(m < 1e300)) m = 1.0;
  double mv = m / fabs(twoR);
  mv = mv * mv;
  if (!(mv > 0.0) || !(mv < 1e300)) mv = 1.0;
  auto expo = [](double room) {  // ilogb: the exact floor(log2(room))
    const int e = ilogb(room);
    return e > 60 ? 60 : (e < -100 ? -100 : e);
  };
  const int Ssp = expo(1073741824.0 / m), Sdd = expo(16777216.0 / m), Svr = expo(1073741824.0 / mv);
  Scales sc;
  sc.sd_dd = ldexp(1.0, Sdd);
  sc.sd_sp = ldexp(1.0, Ssp);
  sc.sd_vr = ldexp(1.0, Svr);
  sc.sc_dd = (float)sc.sd_dd;
  sc.sc_sp = (float)sc.sd_sp;
  sc.c_vr = (float)(ldexp(1.0, Svr - 2 * Ssp) / (twoR * twoR));  // (tp / 2^Ssp / twoR)^2 * 2^Svr = tp^2 * c_vr
  sc.inv_dd = ldexp(1.0, -Sdd);
  sc.inv_sp = ldexp(1.0, -Ssp);
  sc.inv_vr = ldexp(1.0, -Svr);
  sc.e128 = fix128_exponent(m);
  sc.e128v = fix128_exponent(mv);
  sc.inv128 = ldexp(1.0, -sc.e128);
  sc.inv128v = ldexp(1.0, -sc.e128v);
  return sc;
}

// 2R of a dataset (twice its responsivity, measure_w_box_jk.py:744).
__device__ inline double dataset_twoR(const RegionStats& reg, int J) { return 2.0 * (reg.s1[J] / reg.s2[J]); }

// Kernel parameters passed by value.
struct Params {
  int kind, membership, precision, los, ellipticity, want_variance;
  int n_r, n_p, nb, J, n_sub;
  int n_qbreak, n_pbreak;
  double L, halfL;
  float Lf_hi, Lf_lo, halfLf;
  double rp_cut2;               // rp_cut^2 (multipoles), exact decision uses rp > rp_cut via q_p
  double rp_cut;
  // cell grids: shapes on the coarse grid (n, s, R), positions on the fine grid (nf, sf, Rf)
  int axis[3], n[3], R[3], full[3], m[3], nf[3], Rf[3];
  double s[3], inv_s[3], sf[3];
  double range_proj, range_los;
  long long n_cells;
  int shapes_per_unit;
  int reg_slots;                // work units per run of shapes: the most jackknife regions a neighbourhood touches
  // mixed-form guards and tables
  int lut32_base;               // bucket of the first lut32 entry
  float p_lo32, p_inv32;        // Pi/mu: t = (v - p_lo) * p_inv, bin = floor(t)
  float p_off32;                // -p_lo * p_inv: t = fma(v, p_inv, p_off)
  float p_guard;                // fraction of a bin treated as ambiguous at each edge
  float p_half_in;              // 0.5 - p_guard: |frac(t) - 0.5| above it is an edge
  float p_guard_w;              // short w path: |t - rint(t)| below it is an edge (t from the shape's hi/lo z)
  int short_ok;                 // the short pair path applies (finite q_cut inside the lookup table)
  int short_wrap;               // w whose line-of-sight reach spans the box, Pi range inside [-L/2, L/2]:
                                // the short path with a per-pair minimum image along the line of sight
  float t_wrap_lo, t_wrap_hi;   // that path: Pi bin coordinates of -L/2 and L/2 (the wrap points)
  float L_t;                    // that path: L in bin-coordinate units, L n_p / (p_hi - p_lo)
  float c_guard;                // sin^2(phi) below which the exact FP64 cos(phi) decides
  float wrap_guard;
  float los_cut;                // |Pi| above this is surely outside the Pi bins (w)
  float zwin;                   // half-width of the line-of-sight window over the LOS-sorted shapes
  float range_los32;            // range_los in FP32: zwin - range_los32 is the window's slack
  float q_cut;                  // q above this is surely beyond the last binned separation
  float pre_margin;             // FP64 form: bound on the FP32 error of a separation from single floats
  long long edge_capacity;
};

// Workspace pointers, derived from a Plan and a base address.
struct Work {
  Status* status;
  Tables* tables;
  int *pcount, *pstart, *pcur, *scount, *sstart, *scur_lo, *scur_hi;
  int *wucount, *wustart, *tiles;
  int *pcell, *plab, *scell, *slab;
  // sorted positions: FP64 coordinates in cell-dimension order and weights
  double *px, *py, *pz, *pw;
  int* plab_s;
  // mixed form: FP32 hi/lo coordinates and weight
  float *pxh, *pxl, *pyh, *pyl, *pzh, *pzl, *pwf;
  // sorted shapes
  double *sx, *sy, *sz, *sax, *say, *se, *sws;
  int* slab_s;
  float *sxh, *sxl, *syh, *syl, *szh, *szl, *saxf, *sayf, *swef, *swsf;
  WorkUnit* wu;
  RegionStats reg;
  int2* edges;
  // exact fixed-point sums of every pair's terms, in the dataset's scales
  // (dataset_scales): w and S+D for all pairs and each jackknife region
  // ((1+J) * nb), SxD and the variance terms (nb).  Mixed form: one 64-bit
  // word per sum; FP64 form: two (Fix128 lo, hi) per sum
  long long *acc_dd, *acc_sp, *acc_sx, *acc_vr;
  long long edge_capacity;
};

// Output pointers (into the caller's result buffers).
struct Out {
  double* dd;        // (1+J) * nb
  double* splus;     // (1+J) * nb
  double* scross;    // nb
  double* variance;  // nb
  unsigned long long* npairs;   // (1+J) * nb
};

// One dataset of a batch: its workspace and its outputs.
struct Dataset {
  Work w;
  Out o;
};

// Batch header at the start of a (batch) workspace.
struct BatchHeader {
  unsigned long long wu_next;   // global work counter of the pair kernel
  unsigned flags;               // OR of the datasets' status flags (after mia_batch_status)
  int first_bad;                // first dataset with a range error
  unsigned long long bad_index;
  unsigned long long pad[5];
};

// --------------------------------------------------------------------------
// Exact FP64 pair arithmetic: the reference's per-pair sequence of IEEE
// operations (measure_w_box_jk.py:584-617, measure_m_box_jk.py:611-653),
// written with explicit round-to-nearest intrinsics so that no operation is
// fused into an FMA.
// --------------------------------------------------------------------------

// Signed doubles mapped to integers in value order.
__host__ __device__ inline long long order_key(double v) {
#ifdef __CUDA_ARCH__
  long long b = __double_as_longlong(v);
#else
  long long b;
  memcpy(&b, &v, 8);
#endif
  return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b) - 1;
}

__device__ __forceinline__ double wrap_exact(double d, double L, double halfL) {
  // sep[sep > L/2] -= L ; sep[sep < -L/2] += L   (measure_w_box_jk.py:585-587)
  if (d > halfL) d = __dsub_rn(d, L);
  if (d < -halfL) d = __dadd_rn(d, L);
  return d;
}

// Number of breakpoints <= key (binary search over an ascending key table).
__device__ __forceinline__ int count_le(const long long* keys, int n, long long key) {
  int lo = 0, hi = n;  // answer in [lo, hi]
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (keys[mid] <= key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

struct PairResult {
  int bin;      // -1 if not binned
  double ep;    // e cos 2phi (0 under the reference's NaN rule)
  double ex;    // e sin 2phi
};

// Shape s, position p: coordinates in cell-dimension order (d0, d1 projected,
// d2 line of sight).  `perm_r2` selects the original-axis order of the 3-D sum.
template <class Tab>  // Tables in global memory, or the kernel's shared-memory copy of its keys and bins
__device__ __forceinline__ PairResult pair_exact(const Params& P, const Tab& T, double sx, double sy,
                                                 double sz, double ax, double ay, double e, double qx, double qy,
                                                 double qz) {
  PairResult res;
  res.bin = -1;
  res.ep = 0.0;
  res.ex = 0.0;
  double dx = wrap_exact(__dsub_rn(sx, qx), P.L, P.halfL);
  double dy = wrap_exact(__dsub_rn(sy, qy), P.L, P.halfL);
  double dz = wrap_exact(__dsub_rn(sz, qz), P.L, P.halfL);
  double xx = __dmul_rn(dx, dx), yy = __dmul_rn(dy, dy), zz = __dmul_rn(dz, dz);
  double qp = __dadd_rn(xx, yy);  // r_p^2 = sum over not-LOS axes in axis order
  double q;
  if (P.kind == MIA_KIND_W) {
    q = qp;
  } else {
    // r^2 = (s_x^2 + s_y^2) + s_z^2 in ORIGINAL axis order; (d0, d1, d2) is
    // (x, y, z) for LOS 2, (y, z, x) for LOS 0 and (x, z, y) for LOS 1
    if (P.los == 2) q = __dadd_rn(__dadd_rn(xx, yy), zz);
    else if (P.los == 0) q = __dadd_rn(__dadd_rn(zz, xx), yy);
    else q = __dadd_rn(__dadd_rn(xx, zz), yy);
  }
  int ib = T.q_bin[count_le(T.q_key, P.n_qbreak, __double_as_longlong(q))];
  if (ib < 0) return res;
  int jb;
  if (P.kind == MIA_KIND_W) {
    jb = T.p_bin[count_le(T.p_key, P.n_pbreak, order_key(dz))];
  } else {
    // r_p > rp_cut (for rp_cut = 0 that is r_p^2 > 0, no square root needed)
    if (P.rp_cut == 0.0 ? !(qp > 0.0) : !(__dsqrt_rn(qp) > P.rp_cut)) return res;
    double r = __dsqrt_rn(q);
    double mu = __ddiv_rn(dz, r);
    jb = T.p_bin[count_le(T.p_key, P.n_pbreak, order_key(mu))];
  }
  if (jb < 0) return res;
  res.bin = ib * P.n_p + jb;
  // phi = arccos(sdir . a) with sdir = proj / r_p (measure_w_box_jk.py:590-596),
  // e+ = e cos 2phi, ex = e sin 2phi.  With the unit axis a, dot = d . a and
  // crs = d x a: cos 2phi = (dot^2 - crs^2) / r_p^2, sin 2phi = 2 dot |crs| /
  // r_p^2, a short chain within a few ulps of the reference's arccos route.
  // That route runs as written where it is ill-conditioned or takes its NaN
  // rule: sin^2 phi below 1e-6 (c near +-1, where (1 - c)(1 + c) cancels and
  // |c| > 1 can occur), r_p = 0, a NaN axis (the comparison below is false).
  const double dot = fma(dx, ax, dy * ay), crs = fma(dx, ay, -(dy * ax));
  const double s2 = crs * crs;
  if (s2 >= 1e-6 * qp && qp > 0.0) {
    const double f = e / qp;
    res.ep = fma(dot, dot, -s2) * f;
    res.ex = 2.0 * dot * fabs(crs) * f;
    return res;
  }
  const double rp = __dsqrt_rn(qp);
  double c = __dadd_rn(__dmul_rn(__ddiv_rn(dx, rp), ax), __dmul_rn(__ddiv_rn(dy, rp), ay));
  if (c >= -1.0 && c <= 1.0) {  // arccos of |c| > 1 (or NaN) is NaN -> e_+ = e_x = 0
    double c2 = __dmul_rn(c, c);
    double cos2 = __dsub_rn(__dadd_rn(c2, c2), 1.0);
    double s = __dsqrt_rn(__dmul_rn(__dsub_rn(1.0, c), __dadd_rn(1.0, c)));
    double sin2 = __dmul_rn(__dadd_rn(c, c), s);
    res.ep = __dmul_rn(e, cos2);
    res.ex = __dmul_rn(e, sin2);
  }
  return res;
}

// Workspace carve-up (host); returns false on a bad configuration.
bool make_plan(const mia_config* cfg, long long n_pos, long long n_shape, Plan* plan, const char** why);
void bind_work(const Plan& plan, void* base, Work* w);

// Stage launchers (mia_prep.cu, mia_pairs.cu, mia_post.cu)
cudaError_t launch_prep(const Plan& plan, const Params& P, const mia_catalog& cat, const Work& w, cudaStream_t st);
cudaError_t launch_pairs(const Params& P, const Dataset* ds_dev, int n_ds, const unsigned long long* wu_prefix,
                         unsigned long long* wu_next, cudaStream_t st, int num_sms);
cudaError_t launch_edge_retest(const Params& P, const Work& w, const Out& o, cudaStream_t st, int num_sms);
cudaError_t launch_batch_prefix(const Dataset* ds_dev, int n_ds, int reg_slots, unsigned long long* wu_prefix,
                                cudaStream_t st);
cudaError_t launch_post(const Params& P, const Work& w, const mia_layout& lay, double* out, double volume,
                        long long n_pos, long long n_shape, cudaStream_t st);
cudaError_t launch_fixed_out(const Params& P, const Work& w, const Out& o, cudaStream_t st);
// Lightcone pair counts (mia_lightcone.cu): workspace plan and launcher.
struct LcPlan {
  long long n_cells;
  int n_tiles, Q, hq, nb, P, warps, wide;
  size_t smem;
  size_t off_scount, off_sstart, off_sfill, off_pcount, off_pstart, off_pfill, off_tiles, off_scell, off_pcell;
  size_t off_shp, off_pos, off_A, off_B, off_cA, off_cB, off_A128, off_B128, off_wmax, off_win, off_next, total;
};
bool lc_plan(const mia_lc_config* cfg, long long n_pos, long long n_shape, LcPlan* plan, const char** why);
cudaError_t launch_lc(const mia_lc_config* cfg, const LcPlan& plan, const mia_lc_sample& pos,
                      const mia_lc_sample& shp, void* workspace, double* out, int64_t* counts, uint32_t* status,
                      int num_sms, cudaStream_t st);
// exclusive prefix sum of n ints into out[0..n] (out[n] = total), tiles: (n / kScanTile + 1) ints
cudaError_t exclusive_scan(const int* in, long long n, int* out, int* tiles, cudaStream_t st);

cudaError_t launch_cross_cov(int n_real, int n_bins, const double* a, long long sa, const double* b, long long sb,
                             double* cov, double* std, cudaStream_t st);

}  // namespace mia
