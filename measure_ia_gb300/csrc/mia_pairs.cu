// Pair-counting kernels: the persistent cell-pair kernel in its plain FP64 and
// mixed FP32 forms, and the FP64 re-test of near-edge pairs.
//
// Reference hot loop replaced: the per-shape pair binning and np.add.at
// scatters of _measure_xi_rp_pi_box_jk_batch (measure_w_box_jk.py:581-644) and
// _measure_xi_r_mur_box_jk_batch (measure_m_box_jk.py:608-680), together with
// the KD-tree candidate search that feeds them (:577-580) and the Pool.map over
// shape chunks (:765-780).
//
// Work decomposition: a run is up to `shapes_per_unit` shapes of one cell
// that share a jackknife label a; a work unit is one run together with one
// jackknife region b of the positions around it (the regions a run's
// neighbourhood touches are enumerated per unit; without a jackknife every
// run is one unit).  A block takes a unit from a global counter, stages the
// shapes in shared memory, and streams the positions of region b in the
// neighbouring cells (rows of cells along d0 are contiguous in the sorted
// position arrays; cells refine the sub-box grid, so a row clipped to b's
// range is one index range); each thread owns one position at a time and
// loops over the unit's shapes.  Pair contributions go to one block-private
// shared histogram, which each lane of a warp updates in its own copy, and
// are flushed at the end of the unit into the global histograms of all
// pairs, of region a and of region b != a (the attribution rule of
// measure_w_box_jk.py:625-644).  A position whose label is not b (a point on
// a sub-box face carries label 0 wherever it is) adds its pairs to the
// global sums directly.
//
// Sums are exact integers in both forms, so no result depends on the order in
// which blocks meet the pairs: the mixed form adds FP32 terms as 64-bit fixed
// point (32-bit low words with carries), the FP64 form adds FP64 terms as
// 128-bit fixed point (Fix128); one kernel converts each sum to a double at
// the end.
#include <cstdio>

#include "mia_internal.cuh"


namespace mia {

namespace {


constexpr int kRowsPerPass = 256;
constexpr int kSegsPerPass = 2 * kRowsPerPass;

struct SmemLayout {
  size_t tables, shapes, seg_begin, seg_pref, seg_shift, wpos, ring, hist, total;
};

// FP64 form, per warp: a ring of kRing candidate pairs (shape << 5 | lane)
// that passed the range test.
constexpr int kRing = 64;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// u32 words of histogram state.  hw: words per replicated array (slots x
// bins x private copies); knb: slots x bins.
//   mixed: cnt, dd lo, sp lo, sx lo (+ var lo) replicated; the high words of
//          the 64-bit sums (dd, sp, sx (+ var)) once per (slot, bin): only
//          carries reach them, so they need no copies
//   fp64 : cnt (u32) + dd, sp, sx (+ var) 128-bit sums (Fix128), hw = knb
__host__ __device__ inline size_t hist_u32_words(int hw, int knb, int mixed, int var) {
  if (mixed) return (size_t)hw * (4 + var) + (size_t)knb * (3 + var);
  return (size_t)hw * (1 + 4 * (3 + var)) + 4;
}

struct TablesSmem {
  union {
    struct {  // FP64 form: the breakpoint keys
      long long q_key[MIA_MAX_BREAKS];
      long long p_key[MIA_MAX_BREAKS];
    };
    float4 qdirty[MIA_MAX_BREAKS];  // short mixed path: the guard bands of lutw's buckets
  };
  int q_bin[MIA_MAX_BREAKS + 1];
  float q_lo32[MIA_MAX_BREAKS];
  float q_hi32[MIA_MAX_BREAKS];
  int p_bin[MIA_MAX_BREAKS + 1];
  unsigned short lut32[kLut];
};

__host__ __device__ inline SmemLayout smem_layout(int spu, int hw, int knb, int mixed, int var) {
  SmemLayout L;
  size_t o = 0;
  L.tables = o;
  o = align16(o + sizeof(TablesSmem));
  L.shapes = o;
  o = align16(o + (size_t)spu * (mixed ? 48 : 68));
  L.seg_begin = o;
  o = align16(o + sizeof(int) * kSegsPerPass);
  L.seg_pref = o;
  o = align16(o + sizeof(int) * (kSegsPerPass + 1));
  L.seg_shift = o;
  o = align16(o + sizeof(unsigned char) * kSegsPerPass);
  // FP64 form, two-phase loop: the lanes' positions (two double2 and a label
  // each) and the survivor rings
  L.wpos = o;
  o = align16(o + (mixed ? 0 : sizeof(double2) * 2 * kThreads + sizeof(int) * kThreads));
  L.ring = o;
  o = align16(o + (mixed ? 0 : sizeof(unsigned short) * kRing * (kThreads / 32)));
  L.hist = o;
  o = align16(o + sizeof(unsigned) * hist_u32_words(hw, knb, mixed, var) + 16);
  L.total = o;
  return L;
}

// ---- accumulation helpers ---------------------------------------------------

// 64-bit fixed-point sums built from native 32-bit shared atomics: the low
// word (in a lane's private copy) is a signed 32-bit partial that takes the
// value; when adding v overflows it (it wraps by 2^32) the bin's one high word
// takes +1 or -1.  The sum of a bin is the sum over copies of the signed low
// words plus 2^32 times the high word.  overflow_of is negative exactly when
// adding v to a low word that held `old` overflowed.
__device__ __forceinline__ int overflow_of(unsigned old, int v) {
  const unsigned nw = old + (unsigned)v;
  return (int)((old ^ nw) & ((unsigned)v ^ nw));
}



// Global accumulation of one pair in the mixed form (no slot for its position
// region, or decided by the FP64 re-test): count plus fixed-point terms into
// the dataset's 64-bit sums, for all pairs, region a and region b != a.
__device__ __forceinline__ void acc_global_fixed(const Work& w, const Out& o, int nb, int J, int a, int b, int bin,
                                                 long long vd, long long vp, long long vx, long long vv,
                                                 int want_var) {
  typedef unsigned long long u64;
  atomicAdd(&o.npairs[bin], 1ULL);
  atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[bin]), (u64)vd);
  atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[bin]), (u64)vp);
  atomicAdd(reinterpret_cast<u64*>(&w.acc_sx[bin]), (u64)vx);
  if (want_var) atomicAdd(reinterpret_cast<u64*>(&w.acc_vr[bin]), (u64)vv);
  if (J > 0) {
    const size_t ia = (size_t)(1 + a) * nb + bin;
    atomicAdd(&o.npairs[ia], 1ULL);
    atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[ia]), (u64)vd);
    atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[ia]), (u64)vp);
    if (b != a) {
      const size_t ib = (size_t)(1 + b) * nb + bin;
      atomicAdd(&o.npairs[ib], 1ULL);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[ib]), (u64)vd);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[ib]), (u64)vp);
    }
  }
}

// One term of the FP64 form into a dataset sum: its 128-bit fixed-point value
// into acc[2 i], or, when the term is not finite, the term itself into the
// output double out[i] (which the sums are added to at the end).
__device__ __forceinline__ void add_term(long long* acc, double* out, size_t i, double v, int E) {
  Fix128 f;
  if (to_fix128(v, E, f))
    add_fix128(reinterpret_cast<unsigned long long*>(acc) + 2 * i, f);
  else
    atomicAdd(&out[i], v);
}

// Direct global accumulation in the plain FP64 form (pairs whose position
// region has no slot, or with a term that is not finite): count plus exact
// 128-bit sums, for all pairs, region a and region b != a.
__device__ __forceinline__ void acc_global(const Work& w, const Out& o, const Scales& sc, int nb, int J, int a, int b,
                                           int bin, double dd, double sp, double sx, double var, int want_var) {
  const int E = sc.e128;
  atomicAdd(&o.npairs[bin], 1ULL);
  add_term(w.acc_dd, o.dd, bin, dd, E);
  add_term(w.acc_sp, o.splus, bin, sp, E);
  add_term(w.acc_sx, o.scross, bin, sx, E);
  if (want_var) add_term(w.acc_vr, o.variance, bin, var, sc.e128v);
  if (J > 0) {
    size_t ia = (size_t)(1 + a) * nb + bin;
    atomicAdd(&o.npairs[ia], 1ULL);
    add_term(w.acc_dd, o.dd, ia, dd, E);
    add_term(w.acc_sp, o.splus, ia, sp, E);
    if (b != a) {
      size_t ib = (size_t)(1 + b) * nb + bin;
      atomicAdd(&o.npairs[ib], 1ULL);
      add_term(w.acc_dd, o.dd, ib, dd, E);
      add_term(w.acc_sp, o.splus, ib, sp, E);
    }
  }
}

__device__ __forceinline__ int wrapi(int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); }

// Add a hi/lo float pair and a shift of sh*L (sh in {-1,0,1}) without losing
// the low-order bits: TwoSum on the high parts.
__device__ __forceinline__ void shift_hilo(float& h, float& l, int sh, float Lh, float Ll) {
  if (sh == 0) return;
  float a = h, b = sh > 0 ? Lh : -Lh;
  float s = a + b;
  float bb = s - a;
  float err = (a - (s - bb)) + (b - bb);
  h = s;
  l = l + err + (sh > 0 ? Ll : -Ll);
}

// ---- mixed-form pair processing -----------------------------------------------

struct HistView {
  unsigned* cnt;
  unsigned *dd_lo, *sp_lo, *sx_lo, *vr_lo;
  int *dd_hi, *sp_hi, *sx_hi, *vr_hi;
};

// One position in FP32 hi/lo form, moved to the periodic image of its row.
struct MixedPos {
  float xh, xl, yh, yl, zh, zl, w;
  float loff;  // short w path: -(p_lo + z) n_p / (p_hi - p_lo)
  float2 nh, nl, w2;  // short path: -(x_hi, y_hi), -(x_lo, y_lo), (w, w) as register pairs
  float2 nz;          // short multipole path: -(z_hi, z_lo)
  int idx, lab, slot, base, hbase;
  bool valid;
};

__device__ __forceinline__ void load_mixed_pos(const Params& P, const Work& w, const int* seg_begin,
                                               const int* seg_pref, const unsigned char* seg_shift, int region,
                                               int t, int total, int& seg, MixedPos& p) {
  p.valid = t < total;
  int pidx = 0;
  int code = 13;  // no shift
  if (p.valid) {
    while (t >= seg_pref[seg + 1]) ++seg;
    pidx = seg_begin[seg] + (t - seg_pref[seg]);
    code = seg_shift[seg];
  }
  p.idx = pidx;
  p.lab = p.valid ? w.plab_s[pidx] : region;
  p.slot = p.lab == region ? 0 : -1;
  p.base = 0;
  p.hbase = 0;
  p.xh = w.pxh[pidx]; p.xl = w.pxl[pidx];
  p.yh = w.pyh[pidx]; p.yl = w.pyl[pidx];
  p.zh = w.pzh[pidx]; p.zl = w.pzl[pidx];
  p.w = w.pwf[pidx];
  shift_hilo(p.xh, p.xl, code % 3 - 1, P.Lf_hi, P.Lf_lo);
  shift_hilo(p.yh, p.yl, (code / 3) % 3 - 1, P.Lf_hi, P.Lf_lo);
  shift_hilo(p.zh, p.zl, code / 9 - 1, P.Lf_hi, P.Lf_lo);
}

// Widen [lo, hi) by the shapes whose staged line-of-sight coordinate lies in
// [z - win, z + win] (Z ascending).
__device__ __forceinline__ void z_window(const float* Z, int S, float z, float win, int& lo_out, int& hi_out) {
  const float zlo = z - win, zhi = z + win;
  int lo = 0, hi = S;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (Z[mid] < zlo) lo = mid + 1; else hi = mid;
  }
  const int first = lo;
  hi = S;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (Z[mid] <= zhi) lo = mid + 1; else hi = mid;
  }
  if (first < lo_out) lo_out = first;
  if (lo > hi_out) hi_out = lo;
}

// Everything one (shape i, position p) pair contributes in the mixed form:
// FP32 separations, guarded bin decisions, e+/ex, fixed-point accumulation; a
// pair near any decision edge is queued for the FP64 re-test instead.
// SLOTS: 1 when every position of the warp belongs to the unit's region (no
// per-pair check of the position's slot), 0 otherwise.
template <int KIND, int FULL, int VAR, int SLOTS>
__device__ __forceinline__ void mixed_pair(const Params& P, const TablesSmem& T, const float4& a, const float4& b,
                                           const float2* C, const int* I, int i, const MixedPos& p,
                                           const HistView& h, const Work& w, const Out& o,
                                           const Scales& sc, double twoR, int label_a,
                                           unsigned long long& my_binned) {
  float dz = (a.z - p.zh) + (b.z - p.zl);
  bool edge = false;
  if (FULL) {
    if (KIND == MIA_KIND_W) {
      if (P.full[2]) {
        if (dz > P.halfLf) dz -= P.Lf_hi;
        else if (dz < -P.halfLf) dz += P.Lf_hi;
      }
    } else if (P.full[2] && fabsf(dz) >= P.halfLf - P.wrap_guard) {
      edge = true;
    }
  }
  // early rejection on the line of sight: surely outside [pi_bins[0], pi_bins[-1]]
  if (KIND == MIA_KIND_W && fabsf(dz) > P.los_cut) return;
  const float dx = (a.x - p.xh) + (b.x - p.xl);
  const float dy = (a.y - p.yh) + (b.y - p.yl);
  if (FULL) {
    // pairs whose nearest image differs from the cell image: FP64 decides
    if (P.full[0] && fabsf(dx) >= P.halfLf - P.wrap_guard) edge = true;
    if (P.full[1] && fabsf(dy) >= P.halfLf - P.wrap_guard) edge = true;
  }
  const float qp = fmaf(dx, dx, dy * dy);
  const float q = KIND == MIA_KIND_W ? qp : fmaf(dz, dz, qp);
  // early rejection: surely beyond the last binned separation
  if (q > P.q_cut) return;
  // r bin: logarithmic bucket of q; clean buckets hold the bin itself, buckets
  // touching a guard band fall back to the FP32 guard bands of the breakpoints
  // (a floor(a log2 q + b) form for logarithmic bins measured slower)
  int ib;
  {
    const int bucket = (int)(__float_as_uint(q) >> (23 - kLutMantBits)) - P.lut32_base;
    const unsigned short e = (bucket >= 0 && bucket < kLut) ? T.lut32[bucket] : (unsigned short)0x8000;
    if (!(e & 0x8000)) {
      ib = (int)e - 1;
    } else {
      int iv = e & 0x7fff;
      while (iv < P.n_qbreak && q >= T.q_hi32[iv]) ++iv;
      if (iv < P.n_qbreak && q >= T.q_lo32[iv]) edge = true;
      ib = T.q_bin[iv];
    }
  }
  if (ib < 0 && !edge) return;
  int jb;
  {
    float v;
    if (KIND == MIA_KIND_W) {
      v = dz;
    } else {
      if (P.rp_cut2 == 0.0) {
        if (!(qp > 0.0f) && !edge) return;  // r_p > rp_cut = 0 (measure_m_box_jk.py:637)
      } else {
        const float rc2 = (float)P.rp_cut2;
        if (qp < rc2 * (1.0f - 1e-5f)) {
          if (!edge) return;
        } else if (qp <= rc2 * (1.0f + 1e-5f)) {
          edge = true;
        }
      }
      v = dz * rsqrtf(q);
    }
    // t = (v - p_lo) n / (p_hi - p_lo) as one FMA; its fraction within 4x
    // its error bound of 0 or 1 is an edge
    const float t2 = fmaf(v, P.p_inv32, P.p_off32);
    const float fl = floorf(t2);
    jb = (int)fl;
    if (fabsf((t2 - fl) - 0.5f) > P.p_half_in) edge = true;
  }
  if (!edge && (unsigned)jb >= (unsigned)P.n_p) return;
  const float2 cxy = C[i];
  const float dot = fmaf(dx, cxy.x, dy * cxy.y);
  const float crs = fmaf(dx, cxy.y, -dy * cxy.x);
  const float crs2 = crs * crs;
  if (crs2 < P.c_guard * qp) edge = true;
  if (edge) {
    const unsigned long long k = atomicAdd(&w.status->edge_count, 1ULL);
    if (k < (unsigned long long)w.edge_capacity) w.edges[k] = make_int2(I[i], p.idx);
    else atomicOr(&w.status->flags, kStatusOverflow);
    return;
  }
  const int bin = ib * P.n_p + jb;
  // e+ w = w e cos 2phi = w e (dot^2 - crs^2) / r_p^2, ex w = w e 2 dot |crs| / r_p^2
  const float ww = p.w * a.w;                  // scaled by sc_dd
  const float s = __fdividef(p.w * b.w, qp);   // w_p w_s e / r_p^2, scaled by sc_sp
  const float tp = fmaf(dot, dot, -crs2) * s;
  const float tx = (dot * fabsf(crs)) * (s + s);
  if (SLOTS || p.slot >= 0) {  // (binned pairs in the shared histograms are counted at the flush)
    const int k = p.base + bin;
    const int vd = __float2int_rn(ww);
    const int vp = __float2int_rn(tp);
    const int vx = __float2int_rn(tx);
    int vv = 0;
    if (VAR) vv = __float2int_rn(tp * tp * sc.c_vr);
    // low words first (independent atomics), then one rarely taken branch for
    // the overflows into the high words
    const unsigned od = atomicAdd(&h.dd_lo[k], (unsigned)vd);
    const unsigned op = atomicAdd(&h.sp_lo[k], (unsigned)vp);
    const unsigned ox = atomicAdd(&h.sx_lo[k], (unsigned)vx);
    unsigned ov = 0;
    if (VAR) ov = atomicAdd(&h.vr_lo[k], (unsigned)vv);
    atomicAdd(&h.cnt[k], 1u);
    const int fd = overflow_of(od, vd), fp = overflow_of(op, vp), fx = overflow_of(ox, vx);
    const int fv = VAR ? overflow_of(ov, vv) : 0;
    if ((fd | fp | fx | fv) < 0) {
      const int kh = p.hbase + bin;
      if (fd < 0) atomicAdd(&h.dd_hi[kh], (vd >> 31) | 1);
      if (fp < 0) atomicAdd(&h.sp_hi[kh], (vp >> 31) | 1);
      if (fx < 0) atomicAdd(&h.sx_hi[kh], (vx >> 31) | 1);
      if (VAR && fv < 0) atomicAdd(&h.vr_hi[kh], (vv >> 31) | 1);
    }
  } else {
    acc_global_fixed(w, o, P.nb, P.J, label_a, p.lab, bin, __float2ll_rn(ww), __float2ll_rn(tp), __float2ll_rn(tx),
                     VAR ? __float2ll_rn(tp * tp * sc.c_vr) : 0, VAR);
    atomicOr(&w.status->flags, kStatusNoSlot);
    ++my_binned;
  }
}

// The short pair path of the mixed form (local neighbourhoods; w and
// multipoles, with or without variance terms): the same decisions as
// mixed_pair in fewer instructions.
//  * Pi bin: t = (Pi - p_lo) n_p / (p_hi - p_lo) as the shape's staged
//    z n_p / (p_hi - p_lo) plus the position's offset p.loff, bin =
//    floor(t); t within p_guard_w of an integer is an edge.  No separate
//    line-of-sight cut: a pair outside the Pi range has its bin outside
//    [0, n_p).
//  * r bin: the lutw bucket of q holds ib * n_p, kLutReject, or (for a
//    bucket touching a guard band) that band with the codes below and above
//    it; one test covers a reject, a band and a Pi bin outside the range.
//  * Histogram words sit kHistShort (kHistShortVar with variance terms) words
//    apart, so one address serves the four (five) atomics.  `hk` is the lane's
//    copy of the unit's histogram, `hh` the high words.
//  * Paired FP32 instructions (FADD2, FMUL2) where both halves have the same
//    operation: the staged shape is a = (x_hi, y_hi, x_lo, y_lo), b = (z
//    term, z_lo, w_s, w_s e) (scaled weights; the z term is z n_p / (p_hi -
//    p_lo) for w, z_hi for multipoles), so (dx, dy) and the two weight
//    products come out of register pairs; each half rounds as the scalar
//    operation would.
//  * w (mixed_pair_short_w): every rare decision (a reject, a guard-band
//    bucket, a Pi bin outside the range, an edge) sits in one region, so that
//    the common path has a single branch around it; one divergent region
//    instead of three took the 4M / 1M w step's pair kernel from 88.7 to 87.2
//    ms.  The same for multipoles ran 9% slower, so they keep the sequence of
//    mixed_pair_short_m.
//  * Multipoles (mixed_pair_short_m): mu = Pi rsqrt(r^2) and the generic
//    form's bin coordinate and guard; r_p > rp_cut as the generic form decides
//    it.
//  * WRAP (w whose line-of-sight reach spans the box, as with the default
//    pi_max = L/2): t is brought to the minimum image along the line of sight
//    by adding or subtracting L in bin units beyond the wrap points; those
//    coincide with the Pi range's ends (edges) or lie outside it.

// A pair that goes to the FP64 re-test.
__device__ __forceinline__ void short_queue_edge(const Work& w, int shape, int pos) {
  const unsigned long long k = atomicAdd(&w.status->edge_count, 1ULL);
  if (k < (unsigned long long)w.edge_capacity) w.edges[k] = make_int2(shape, pos);
  else atomicOr(&w.status->flags, kStatusOverflow);
}

// The binned pair's terms into the lane's histogram copy (or, without a slot
// for the position's region, into the dataset's sums).
template <int SLOTS, int VAR>
__device__ __forceinline__ void short_accumulate(const Params& P, int bin, const float4& b, const MixedPos& p,
                                                 float qp, float dot, float crs, float crs2, unsigned* hk, int* hh,
                                                 const Work& w, const Out& o, const Scales& sc, int label_a,
                                                 unsigned long long& my_binned) {
  constexpr int KS = VAR ? kHistShortVar : kHistShort;
  const float2 pw = __fmul2_rn(make_float2(b.z, b.w), p.w2);  // (w_p w_s, w_p w_s e), scaled
  const float ww = pw.x;
  const float s = __fdividef(pw.y, qp);
  const float2 tt = __fmul2_rn(make_float2(fmaf(dot, dot, -crs2), dot * fabsf(crs)), make_float2(s, s + s));
  const float tp = tt.x, tx = tt.y;
  if (SLOTS || p.slot >= 0) {
    const int vd = __float2int_rn(ww);
    const int vp = __float2int_rn(tp);
    const int vx = __float2int_rn(tx);
    int vv = 0;
    if (VAR) vv = __float2int_rn(tp * tp * sc.c_vr);
    unsigned* h = hk + bin;
    const unsigned od = atomicAdd(h + KS, (unsigned)vd);
    const unsigned op = atomicAdd(h + 2 * KS, (unsigned)vp);
    const unsigned ox = atomicAdd(h + 3 * KS, (unsigned)vx);
    unsigned ov = 0;
    if (VAR) ov = atomicAdd(h + 4 * KS, (unsigned)vv);
    atomicAdd(h, 1u);
    const int fd = overflow_of(od, vd), fp = overflow_of(op, vp), fx = overflow_of(ox, vx);
    const int fv = VAR ? overflow_of(ov, vv) : 0;
    if ((fd | fp | fx | fv) < 0) {
      int* g = hh + bin;
      if (fd < 0) atomicAdd(g, (vd >> 31) | 1);
      if (fp < 0) atomicAdd(g + P.nb, (vp >> 31) | 1);
      if (fx < 0) atomicAdd(g + 2 * P.nb, (vx >> 31) | 1);
      if (VAR && fv < 0) atomicAdd(g + 3 * P.nb, (vv >> 31) | 1);
    }
  } else {
    acc_global_fixed(w, o, P.nb, P.J, label_a, p.lab, bin, __float2ll_rn(ww), __float2ll_rn(tp), __float2ll_rn(tx),
                     VAR ? __float2ll_rn(tp * tp * sc.c_vr) : 0, VAR);
    atomicOr(&w.status->flags, kStatusNoSlot);
    ++my_binned;
  }
}

template <int SLOTS, int WRAP, int VAR>
__device__ __forceinline__ void mixed_pair_short_w(const Params& P, const TablesSmem& T, const float4& a,
                                                   const float4& b, const float2* C, const int* I, int i,
                                                   const MixedPos& p, unsigned* hk, int* hh, const Work& w,
                                                   const Out& o, const Scales& sc, int label_a,
                                                   unsigned long long& my_binned) {
  const float2 d = __fadd2_rn(__fadd2_rn(make_float2(a.x, a.y), p.nh), __fadd2_rn(make_float2(a.z, a.w), p.nl));
  const float dx = d.x, dy = d.y;
  const float qp = fmaf(dx, dx, dy * dy);
  float t = b.x + p.loff;
  if (WRAP) t = t >= P.t_wrap_hi ? t - P.L_t : (t < P.t_wrap_lo ? t + P.L_t : t);
  // (q <= q_cut lies in the table; a q below it wraps to the last entry,
  // which holds the bin under the first breakpoint; a q above q_cut, whose
  // entry is not used, is clamped to the table too.  The load is issued
  // before the exit below, so its latency overlaps the branch: 89.9 -> 88.7 ms
  // on the 4M / 1M w step)
  const unsigned bucket = min((__float_as_uint(qp) >> (23 - kLutMantBits)) - (unsigned)P.lut32_base, (unsigned)kLut - 1u);
  int e = T.lut32[bucket];
  // surely beyond the last binned separation (whole warps leave here often)
  if (qp > P.q_cut) return;
  const int jb = __float2int_rd(t);
  const bool pi_edge = fabsf(t - rintf(t)) < P.p_guard_w;
  const float2 cxy = C[i];
  const float dot = fmaf(dx, cxy.x, dy * cxy.y);
  const float crs = fmaf(dx, cxy.y, -dy * cxy.x);
  const float crs2 = crs * crs;
  const bool c_edge = crs2 < P.c_guard * qp;  // direction within the guard of the axis line
  if ((e >= kLutReject) | ((unsigned)jb >= (unsigned)P.n_p) | pi_edge | c_edge) {
    // Pi surely outside the bins (an edge at 0 or n_p goes on to the re-test)
    if ((unsigned)jb >= (unsigned)P.n_p && ((unsigned)jb + 1u > (unsigned)P.n_p + 1u || !pi_edge)) return;
    bool edge = pi_edge | c_edge;
    if (e & 0x8000) {  // a bucket touching a guard band: below, inside (an edge) or above the band
      const float* D = reinterpret_cast<const float*>(&T.qdirty[e & 0x7fff]);
      const bool below = qp < D[0], above = qp >= D[1];
      e = below ? __float_as_int(D[2]) : (above ? __float_as_int(D[3]) : 0);
      edge |= !(below || above);
    }
    if (e == kLutReject) return;
    if (edge) {
      short_queue_edge(w, I[i], p.idx);
      return;
    }
  }
  short_accumulate<SLOTS, VAR>(P, e + jb, b, p, qp, dot, crs, crs2, hk, hh, w, o, sc, label_a, my_binned);
}

template <int SLOTS, int VAR>
__device__ __forceinline__ void mixed_pair_short_m(const Params& P, const TablesSmem& T, const float4& a,
                                                   const float4& b, const float2* C, const int* I, int i,
                                                   const MixedPos& p, unsigned* hk, int* hh, const Work& w,
                                                   const Out& o, const Scales& sc, int label_a,
                                                   unsigned long long& my_binned) {
  const float2 d = __fadd2_rn(__fadd2_rn(make_float2(a.x, a.y), p.nh), __fadd2_rn(make_float2(a.z, a.w), p.nl));
  const float dx = d.x, dy = d.y;
  const float qp = fmaf(dx, dx, dy * dy);
  const float2 zz = __fadd2_rn(make_float2(b.x, b.y), p.nz);  // (z_hi, z_lo) differences
  const float dz = zz.x + zz.y;
  const float q = fmaf(dz, dz, qp);
  // (the table and the early exit as for w)
  const unsigned bucket = min((__float_as_uint(q) >> (23 - kLutMantBits)) - (unsigned)P.lut32_base, (unsigned)kLut - 1u);
  int e = T.lut32[bucket];
  if (q > P.q_cut) return;
  const float t = fmaf(dz * rsqrtf(q), P.p_inv32, P.p_off32);
  const int jb = __float2int_rd(t);
  const bool pi_edge = fabsf(t - rintf(t)) < P.p_guard;
  bool edge = pi_edge;
  if ((e >= kLutReject) | ((unsigned)jb >= (unsigned)P.n_p)) {
    // mu surely outside the bins (an edge at 0 or n_p goes on to the re-test)
    if ((unsigned)jb >= (unsigned)P.n_p && ((unsigned)jb + 1u > (unsigned)P.n_p + 1u || !pi_edge)) return;
    if (e & 0x8000) {  // a bucket touching a guard band: below, inside (an edge) or above the band
      const float* D = reinterpret_cast<const float*>(&T.qdirty[e & 0x7fff]);
      const bool below = q < D[0], above = q >= D[1];
      e = below ? __float_as_int(D[2]) : (above ? __float_as_int(D[3]) : 0);
      edge |= !(below || above);
    }
    if (e == kLutReject) return;
  }
  if (P.rp_cut2 == 0.0) {
    if (!(qp > 0.0f) && !edge) return;  // r_p > rp_cut = 0 (measure_m_box_jk.py:637)
  } else {
    const float rc2 = (float)P.rp_cut2;
    if (qp < rc2 * (1.0f - 1e-5f)) {
      if (!edge) return;
    } else if (qp <= rc2 * (1.0f + 1e-5f)) {
      edge = true;
    }
  }
  const float2 cxy = C[i];
  const float dot = fmaf(dx, cxy.x, dy * cxy.y);
  const float crs = fmaf(dx, cxy.y, -dy * cxy.x);
  const float crs2 = crs * crs;
  if (crs2 < P.c_guard * qp) edge = true;
  if (edge) {
    short_queue_edge(w, I[i], p.idx);
    return;
  }
  short_accumulate<SLOTS, VAR>(P, e + jb, b, p, qp, dot, crs, crs2, hk, hh, w, o, sc, label_a, my_binned);
}

// FP64 form, the two-phase loop's range test from single-float coordinates:
// the minimum-image gap per axis less `m` (a bound on the FP32 error), so that
// a pair it drops is beyond the binned range in the exact arithmetic too.
__device__ __forceinline__ float fp32_gap(float d, float L, float m) {
  const float a = fabsf(d);
  return fmaxf(fminf(a, L - a) - m, 0.0f);
}

template <int KIND>
__device__ __forceinline__ bool in_range_fp64(const Params& P, float sx, float sy, float sz, float px, float py,
                                              float pz) {
  const float m = P.pre_margin, L = P.Lf_hi;
  const float gx = fp32_gap(sx - px, L, m), gy = fp32_gap(sy - py, L, m), gz = fp32_gap(sz - pz, L, m);
  if (KIND == MIA_KIND_W) return !(gz > P.los_cut) && !(fmaf(gx, gx, gy * gy) > P.q_cut);
  return !(fmaf(gz, gz, fmaf(gx, gx, gy * gy)) > P.q_cut);
}

// Sub-boxes (jackknife regions along one cell dimension) that the fine cells
// lo..hi (unwrapped, periodic) fall in, ascending by first appearance; their
// number.  cps = fine cells per sub-box.
__device__ __forceinline__ int subbox_set(int lo, int hi, int nf, int cps, int n_sub, int* set) {
  int cnt = 0;
  for (int u = lo; u <= hi && cnt < n_sub;) {
    const int cc = ((u % nf) + nf) % nf;
    const int sb = cc / cps;
    bool seen = false;
    for (int j = 0; j < cnt; ++j) seen |= set[j] == sb;
    if (!seen) set[cnt++] = sb;
    u += cps - cc % cps;  // the first cell of the next sub-box
  }
  return cnt;
}

// One position against the staged shapes [wlo, whi): the next shape is in
// flight while this pair is processed (index whi at most: still inside the
// staging area); two register sets take turns, so the prefetched shape is
// never copied.
template <int KIND, int FULL, int VAR, int SLOTS, int SHORT>
__device__ __forceinline__ void shape_loop(const Params& P, const TablesSmem& T, const float4* A, const float4* B,
                                           const float2* C, const int* I, int wlo, int whi, const MixedPos& p0,
                                           const HistView& hv, const Work& w, const Out& o, const Scales& sc,
                                           double twoR, int label_a, unsigned long long& my_binned) {
  // (short path: the lane's copy of the histogram and the high words)
  unsigned* const hk = hv.cnt + p0.base;
  int* const hh = hv.dd_hi + p0.hbase;
  auto pair = [&](const float4& a, const float4& b, int i) {
    if (SHORT) {
      if (KIND == MIA_KIND_W)
        mixed_pair_short_w<SLOTS, SHORT == 2, VAR>(P, T, a, b, C, I, i, p0, hk, hh, w, o, sc, label_a, my_binned);
      else
        mixed_pair_short_m<SLOTS, VAR>(P, T, a, b, C, I, i, p0, hk, hh, w, o, sc, label_a, my_binned);
    } else {
      mixed_pair<KIND, FULL, VAR, SLOTS>(P, T, a, b, C, I, i, p0, hv, w, o, sc, twoR, label_a, my_binned);
    }
  };
  float4 a0 = A[wlo], b0 = B[wlo];
  for (int i = wlo;;) {
    const float4 a1 = A[i + 1], b1 = B[i + 1];
    pair(a0, b0, i);
    if (++i >= whi) break;
    a0 = A[i + 1];
    b0 = B[i + 1];
    pair(a1, b1, i);
    if (++i >= whi) break;
  }
}


// ---- the persistent pair kernel ----------------------------------------------

// (a minimum-blocks bound of 4 gives the same 61 registers but code that
// runs 8% slower on the 4M/1M w step; the register count alone allows 4)
template <int MIXED, int VAR, int KIND, int FULL, int SHORT>
// (4 blocks of 256 threads per SM need 64 registers: asked of the multipole
// and FP64 variants, which the compiler otherwise takes to 80 or beyond --
// mixed multipoles 104.0 against 112.7 ms on the 4M/1M step; the mixed w
// kernel reaches 64 unbounded)
#define MIA_PAIR_MINB (MIXED ? (KIND == MIA_KIND_W ? 0 : 4) : 4)
__global__ void __launch_bounds__(kThreads, MIA_PAIR_MINB) k_pairs(
    Params P, const Dataset* __restrict__ ds, int n_ds,
                                                     const unsigned long long* __restrict__ wu_prefix,
                                                     unsigned long long* wu_next, int HW) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x;
  const int nb = P.nb;
  const SmemLayout SL = smem_layout(P.shapes_per_unit, HW, P.nb, MIXED, VAR);
  TablesSmem& T = *reinterpret_cast<TablesSmem*>(smem + SL.tables);
  int* seg_begin = reinterpret_cast<int*>(smem + SL.seg_begin);
  int* seg_pref = reinterpret_cast<int*>(smem + SL.seg_pref);
  unsigned char* seg_shift = reinterpret_cast<unsigned char*>(smem + SL.seg_shift);
  unsigned* hist = reinterpret_cast<unsigned*>(smem + SL.hist);
  float4* wpos = reinterpret_cast<float4*>(smem + SL.wpos);
  unsigned short* ring = reinterpret_cast<unsigned short*>(smem + SL.ring);
  // words per replicated array (the short path's stride is fixed)
  const int KB = SHORT ? (VAR ? kHistShortVar : kHistShort) : HW;

  __shared__ long long s_wu;
  __shared__ int s_ds;
  __shared__ Dataset s_data;        // the current unit's dataset (workspace and outputs)
  __shared__ double s_twoR;
  __shared__ Scales s_sc;
  __shared__ int s_region;          // jackknife region b of the unit's positions (-1: none, skip the unit)
  __shared__ int s_sub[3];          // b's sub-box along d0, d1, d2
  __shared__ int s_copies;
  __shared__ int s_stride;
  __shared__ int s_scan[32];
  __shared__ int s_total;
  __shared__ float s_box[4];  // the unit's shape cell in d0, d1, widened (see the window below)

  // tables -> shared (the same binning for every dataset of a batch)
  {
    const Tables& G = *ds[0].w.tables;
    for (int i = tid; i < MIA_MAX_BREAKS; i += blockDim.x) {
      if (SHORT) {
        T.qdirty[i] = G.qdirty[i];
      } else {
        T.q_key[i] = G.q_key[i];
        T.p_key[i] = G.p_key[i];
      }
      T.q_lo32[i] = G.q_lo32[i];
      T.q_hi32[i] = G.q_hi32[i];
    }
    for (int i = tid; i < MIA_MAX_BREAKS + 1; i += blockDim.x) {
      T.q_bin[i] = G.q_bin[i];
      T.p_bin[i] = G.p_bin[i];
    }
    if (MIXED)
      for (int i = tid; i < kLut; i += blockDim.x) T.lut32[i] = SHORT ? G.lutw[i] : G.lut32[i];
    if (tid == 0) s_ds = -1;
  }
  const unsigned long long n_wu_all = wu_prefix[n_ds];
  __syncthreads();

  // views of the per-bin state
  unsigned* h_cnt = hist;
  unsigned *dd_lo = nullptr, *sp_lo = nullptr, *sx_lo = nullptr, *vr_lo = nullptr;
  int *dd_hi = nullptr, *sp_hi = nullptr, *sx_hi = nullptr, *vr_hi = nullptr;
  unsigned long long *dd_q = nullptr, *sp_q = nullptr, *sx_q = nullptr, *vr_q = nullptr;  // Fix128 pairs
  if (MIXED) {
    dd_lo = hist + KB;
    sp_lo = hist + 2 * KB;
    sx_lo = hist + 3 * KB;
    if (VAR) vr_lo = hist + 4 * KB;
    int* hi = reinterpret_cast<int*>(hist + (4 + VAR) * KB);
    const int knb = nb;
    dd_hi = hi;
    sp_hi = hi + knb;
    sx_hi = hi + 2 * knb;
    if (VAR) vr_hi = hi + 3 * knb;
  } else {
    // 128-bit sums (two 64-bit words each) start at a 16-byte boundary after the counts
    size_t off = align16(sizeof(unsigned) * (size_t)KB);
    unsigned long long* base = reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(hist) + off);
    dd_q = base;
    sp_q = base + 2 * KB;
    sx_q = base + 4 * KB;
    if (VAR) vr_q = base + 6 * KB;
  }
  const int hist_u32 = MIXED ? (int)hist_u32_words(KB, nb, 1, VAR)
                             : (int)(align16(sizeof(unsigned) * (size_t)KB) / 4) + KB * 4 * (3 + VAR);

  // rows of position cells: fine-grid extents along d1 and d2 around a shape cell
  const int N1 = P.full[1] ? P.nf[1] : P.m[1] + 2 * P.Rf[1];
  const int N2 = P.full[2] ? P.nf[2] : P.m[2] + 2 * P.Rf[2];
  const int n_rows = N1 * N2;
  const double r2proj = P.range_proj * P.range_proj;
  const double r2los = P.range_los * P.range_los;

  while (true) {
    // -- the next unit with work, found by one thread: global unit g is slot
    // rslot of run g / reg_slots of its dataset, and that slot is one of the
    // jackknife regions the run's neighbourhood touches (sub-boxes per
    // dimension, all combinations), or past their number (nothing to do, and
    // the thread takes the next unit at once); a catalogue with coordinates
    // outside [0, L) or not finite ends in MIA_ERR_RANGE, so its units are
    // skipped as well
    if (tid == 0) {
      long long found = -1;
      while (true) {
        const unsigned long long g = atomicAdd(wu_next, 1ULL);
        if (g >= n_wu_all) break;
        // dataset of global unit g: largest d with wu_prefix[d] <= g
        int lo = 0, hi = n_ds - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (wu_prefix[mid] <= g) lo = mid; else hi = mid - 1;
        }
        if (lo != s_ds) {
          s_ds = lo;
          s_data = ds[lo];
          const Work& wd = ds[lo].w;
          s_twoR = dataset_twoR(wd.reg, P.J);
          s_sc = dataset_scales(wd.status, s_twoR);
        }
        if (*reinterpret_cast<volatile const unsigned*>(&s_data.w.status->flags) & kStatusRange) continue;
        const long long wi = (long long)(g - wu_prefix[lo]);
        const WorkUnit u = s_data.w.wu[wi / P.reg_slots];
        const int rslot = (int)(wi % P.reg_slots);
        int c[3];
        {
          long long t = u.cell;
          c[0] = (int)(t % P.n[0]);
          t /= P.n[0];
          c[1] = (int)(t % P.n[1]);
          c[2] = (int)(t / P.n[1]);
        }
        int reg = 0;
        s_sub[0] = s_sub[1] = s_sub[2] = 0;
        if (P.J > 0) {
          int sets[3][16], cnt[3];
          for (int k = 0; k < 3; ++k) {
            const int f = c[k] * P.m[k];
            const int a0 = P.full[k] ? 0 : f - P.Rf[k];
            const int a1 = P.full[k] ? P.nf[k] - 1 : f + P.m[k] - 1 + P.Rf[k];
            cnt[k] = subbox_set(a0, a1, P.nf[k], P.nf[k] / P.n_sub, P.n_sub, sets[k]);
          }
          if (rslot >= cnt[0] * cnt[1] * cnt[2]) continue;
          const int i0 = rslot % cnt[0], i1 = (rslot / cnt[0]) % cnt[1], i2 = rslot / (cnt[0] * cnt[1]);
          s_sub[0] = sets[0][i0];
          s_sub[1] = sets[1][i1];
          s_sub[2] = sets[2][i2];
          int sub[3];
          sub[P.axis[0]] = s_sub[0];
          sub[P.axis[1]] = s_sub[1];
          sub[P.axis[2]] = s_sub[2];
          reg = (sub[0] * P.n_sub + sub[1]) * P.n_sub + sub[2];
        } else if (rslot > 0) {
          continue;
        }
        found = wi;
        s_region = reg;
        // the shape cell's projected box, widened by 1e-3 r_max + 1e-5 L: more
        // than the FP32 error of a position's coordinates, so a gap measured
        // to it never exceeds the true gap to any of the cell's shapes
        const double m = 1e-3 * P.range_proj + 1e-5 * P.L;
        s_box[0] = (float)(c[0] * P.s[0] - m);
        s_box[1] = (float)((c[0] + 1) * P.s[0] + m);
        s_box[2] = (float)(c[1] * P.s[1] - m);
        s_box[3] = (float)((c[1] + 1) * P.s[1] + m);
        // private copies of the unit's histogram (mixed form): lanes holding
        // neighbouring positions hit the same bin against a shape, and shared
        // atomics on one address serialise, so lane l adds into copy l mod R;
        // the odd stride puts the R copies of a bin in R distinct banks.  No
        // more copies than the unit has shapes: each copy is zeroed and read
        // back once per unit
        int R = 1;
        const int stride = nb | 1;
        if (MIXED)
          while (R < 32 && R < u.count && (2 * R) * stride <= HW) R *= 2;
        s_copies = R;
        s_stride = R > 1 ? stride : nb;
        break;
      }
      s_wu = found;
    }
    __syncthreads();
    const long long wi = s_wu;
    if (wi < 0) break;
    const Work& w = s_data.w;
    const Out& o = s_data.o;
    const double twoR = s_twoR;
    const Scales& sc = s_sc;
    unsigned long long my_binned = 0;
    const WorkUnit u = w.wu[wi / P.reg_slots];
    int c[3];
    {
      long long t = u.cell;
      c[0] = (int)(t % P.n[0]);
      t /= P.n[0];
      c[1] = (int)(t % P.n[1]);
      c[2] = (int)(t / P.n[1]);
    }
    const int region = s_region;
    if (MIXED) {
      // the copies in use of the replicated words, and the high words
      const int used = s_copies * s_stride;
      for (int i = tid; i < (4 + VAR) * KB + (3 + VAR) * nb; i += blockDim.x)
        if (i >= (4 + VAR) * KB || i % KB < used) hist[i] = 0u;
    } else {
      for (int i = tid; i < hist_u32; i += blockDim.x) hist[i] = 0u;
    }
    // -- shapes of the unit -> shared
    const int S = u.count;
    if (MIXED) {
      // stage the shapes ordered by line-of-sight coordinate: a position then
      // meets only a contiguous window of them within the Pi range
      float4* A = reinterpret_cast<float4*>(smem + SL.shapes);
      float4* B = A + P.shapes_per_unit;
      float2* C = reinterpret_cast<float2*>(B + P.shapes_per_unit);
      int* I = reinterpret_cast<int*>(C + P.shapes_per_unit);
      float* Z = reinterpret_cast<float*>(I + P.shapes_per_unit);
      float* zs = reinterpret_cast<float*>(seg_begin);  // free until the segments are built
      float4 ra = make_float4(0.f, 0.f, 0.f, 0.f), rb = ra;
      float2 rc = make_float2(0.f, 0.f);
      float z = 0.f;
      const int g = u.begin + tid;
      if (tid < S) {
        // weights times the (power-of-two) fixed-point scales: exact; the
        // short path pairs (x, y) hi, (x, y) lo, (z hi, z lo) and the weights
        if (SHORT) {
          // (w: the line-of-sight coordinate times n_p / (p_hi - p_lo) in one
          // float, the shape's share of the Pi bin coordinate)
          ra = make_float4(w.sxh[g], w.syh[g], w.sxl[g], w.syl[g]);
          const float zh = w.szh[g], zl = w.szl[g];
          rb = make_float4(KIND == MIA_KIND_W ? fmaf(zh, P.p_inv32, zl * P.p_inv32) : zh, zl,
                           w.swsf[g] * sc.sc_dd, w.swef[g] * sc.sc_sp);
        } else {
          ra = make_float4(w.sxh[g], w.syh[g], w.szh[g], w.swsf[g] * sc.sc_dd);
          rb = make_float4(w.sxl[g], w.syl[g], w.szl[g], w.swef[g] * sc.sc_sp);
        }
        rc = make_float2(w.saxf[g], w.sayf[g]);
        z = SHORT ? w.szh[g] + w.szl[g] : ra.z + rb.z;
        if (!(z == z)) z = INFINITY;  // the ranks below must form a permutation
        zs[tid] = z;
      }
      __syncthreads();
      if (tid < S) {
        int rank = 0;
        for (int j = 0; j < S; ++j) {
          const float zj = zs[j];
          rank += (zj < z || (zj == z && j < tid)) ? 1 : 0;
        }
        A[rank] = ra;
        B[rank] = rb;
        C[rank] = rc;
        I[rank] = g;
        Z[rank] = z;
      }
    } else {
      // FP64 form: the unit's shapes in line-of-sight order too (the sums are
      // order-free), with their line-of-sight coordinates in FP32 for the window
      double* D = reinterpret_cast<double*>(smem + SL.shapes);
      const int M = P.shapes_per_unit;
      float* Z = reinterpret_cast<float*>(D + 7 * M);
      float* zs = reinterpret_cast<float*>(seg_begin);  // free until the segments are built
      const int g = u.begin + tid;
      float z = 0.f;
      if (tid < S) {
        z = (float)w.sz[g];
        if (!(z == z)) z = INFINITY;  // the ranks below must form a permutation
        zs[tid] = z;
      }
      __syncthreads();
      if (tid < S) {
        int rank = 0;
        for (int j = 0; j < S; ++j) {
          const float zj = zs[j];
          rank += (zj < z || (zj == z && j < tid)) ? 1 : 0;
        }
        D[rank] = w.sx[g];
        D[M + rank] = w.sy[g];
        D[2 * M + rank] = w.sz[g];
        D[3 * M + rank] = w.sax[g];
        D[4 * M + rank] = w.say[g];
        D[5 * M + rank] = w.se[g];
        D[6 * M + rank] = w.sws[g];
        Z[rank] = z;
        Z[M + rank] = (float)w.sx[g];
        Z[2 * M + rank] = (float)w.sy[g];
      }
    }
    __syncthreads();

    for (int pass = 0; pass < n_rows; pass += kRowsPerPass) {
      // -- segments of this pass: two per row (a row may wrap around d0)
      for (int rr = tid; rr < kRowsPerPass; rr += blockDim.x) {
        int r = pass + rr;
        int len0 = 0, len1 = 0, b0 = 0, b1 = 0, sh0 = 0, sh1 = 0;
        if (r < n_rows) {
          // unwrapped fine indices of the row and its distance to the shape cell
          const int f1 = c[1] * P.m[1], f2 = c[2] * P.m[2];
          const int lo1 = P.full[1] ? f1 - (P.nf[1] - P.m[1]) / 2 : f1 - P.Rf[1];
          const int lo2 = P.full[2] ? f2 - (P.nf[2] - P.m[2]) / 2 : f2 - P.Rf[2];
          const int u1 = lo1 + r % N1, u2 = lo2 + r / N1;
          const int g1 = u1 > f1 + P.m[1] - 1 ? u1 - f1 - P.m[1] : (u1 < f1 ? f1 - u1 - 1 : 0);
          const int g2 = u2 > f2 + P.m[2] - 1 ? u2 - f2 - P.m[2] : (u2 < f2 ? f2 - u2 - 1 : 0);
          const double gap1 = g1 * P.sf[1], gap2 = g2 * P.sf[2];
          double rem;
          bool ok;
          if (KIND == MIA_KIND_W) {
            ok = gap1 * gap1 <= r2proj && gap2 * gap2 <= r2los;
            rem = r2proj - gap1 * gap1;
          } else {
            rem = r2proj - gap1 * gap1 - gap2 * gap2;
            ok = rem >= 0.0;
          }
          const int cc1 = wrapi(u1, P.nf[1]), cc2 = wrapi(u2, P.nf[2]);
          // only the cells of the unit's position region
          if (P.J > 0 && ((long long)cc1 * P.n_sub / P.nf[1] != s_sub[1] ||
                          (long long)cc2 * P.n_sub / P.nf[2] != s_sub[2]))
            ok = false;
          if (ok) {
            const int sh1d = u1 < 0 ? -1 : (u1 >= P.nf[1] ? 1 : 0);
            const int sh2d = u2 < 0 ? -1 : (u2 >= P.nf[2] ? 1 : 0);
            const int f0 = c[0] * P.m[0];
            int a0, a1;
            if (P.full[0]) {
              a0 = f0 - (P.nf[0] - P.m[0]) / 2;
              a1 = a0 + P.nf[0] - 1;
            } else {
              int R0 = (int)ceil(sqrt(rem > 0.0 ? rem : 0.0) / P.sf[0] * (1.0 + 1e-9));
              if (R0 > P.Rf[0]) R0 = P.Rf[0];
              a0 = f0 - R0;
              a1 = f0 + P.m[0] - 1 + R0;
            }
            const long long rowbase = ((long long)cc2 * P.nf[1] + cc1) * P.nf[0];
            const int code_yz = 3 * (sh1d + 1) + 9 * (sh2d + 1);
            // the row's cells as at most two wrapped ranges [x0, x1] (d0 shift -1, 0 or +1),
            // each clipped to the unit's region along d0
            int x0a, x1a, x0b = 0, x1b = -1;
            if (a0 < 0) {
              x0a = a0 + P.nf[0];
              x1a = P.nf[0] - 1;
              sh0 = code_yz + 0;  // d0 shift -1
              x0b = 0;
              x1b = a1;
              sh1 = code_yz + 1;
            } else if (a1 >= P.nf[0]) {
              x0a = a0;
              x1a = P.nf[0] - 1;
              sh0 = code_yz + 1;
              x0b = 0;
              x1b = a1 - P.nf[0];
              sh1 = code_yz + 2;  // d0 shift +1
            } else {
              x0a = a0;
              x1a = a1;
              sh0 = code_yz + 1;
            }
            if (P.J > 0) {
              const int cps = P.nf[0] / P.n_sub;
              const int r0 = s_sub[0] * cps, r1 = r0 + cps - 1;
              x0a = max(x0a, r0);
              x1a = min(x1a, r1);
              x0b = max(x0b, r0);
              x1b = min(x1b, r1);
            }
            if (x0a <= x1a) {
              b0 = w.pstart[rowbase + x0a];
              len0 = w.pstart[rowbase + x1a + 1] - b0;
            }
            if (x0b <= x1b) {
              b1 = w.pstart[rowbase + x0b];
              len1 = w.pstart[rowbase + x1b + 1] - b1;
            }
          }
        }
        seg_begin[2 * rr] = b0;
        seg_begin[2 * rr + 1] = b1;
        seg_shift[2 * rr] = (unsigned char)sh0;
        seg_shift[2 * rr + 1] = (unsigned char)sh1;
        seg_pref[2 * rr] = len0;
        seg_pref[2 * rr + 1] = len1;
      }
      __syncthreads();
      // exclusive scan of segment lengths (kSegsPerPass values, 4 per thread)
      {
        constexpr int per = kSegsPerPass / kThreads;
        int v[per], loc = 0;
        for (int k = 0; k < per; ++k) {
          v[k] = seg_pref[tid * per + k];
          loc += v[k];
        }
        int x = loc;
        const int lane = tid & 31, wid = tid >> 5;
        for (int of = 1; of < 32; of <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, x, of);
          if (lane >= of) x += y;
        }
        if (lane == 31) s_scan[wid] = x;
        __syncthreads();
        if (wid == 0) {
          int t = lane < (kThreads / 32) ? s_scan[lane] : 0;
          for (int of = 1; of < 32; of <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, of);
            if (lane >= of) t += y;
          }
          if (lane < (kThreads / 32)) s_scan[lane] = t;
        }
        __syncthreads();
        int ex = (wid > 0 ? s_scan[wid - 1] : 0) + x - loc;
        for (int k = 0; k < per; ++k) {
          seg_pref[tid * per + k] = ex;
          ex += v[k];
        }
        if (tid == kThreads - 1) {
          seg_pref[kSegsPerPass] = ex;
          s_total = ex;
        }
        __syncthreads();
      }
      const int total = s_total;
      if (MIXED) {
        const float4* A = reinterpret_cast<const float4*>(smem + SL.shapes);
        const float4* B = A + P.shapes_per_unit;
        const float2* C = reinterpret_cast<const float2*>(B + P.shapes_per_unit);
        const int* I = reinterpret_cast<const int*>(C + P.shapes_per_unit);
        const float* Z = reinterpret_cast<const float*>(I + P.shapes_per_unit);
        const HistView hv{h_cnt, dd_lo, sp_lo, sx_lo, vr_lo, dd_hi, sp_hi, sx_hi, vr_hi};
        int seg = 0;
        const int copy_off = (tid & (s_copies - 1)) * s_stride;
        // every warp runs the same number of iterations so that its lanes can
        // agree on one shape range
        for (int tb = 0; tb < total; tb += blockDim.x) {
          MixedPos p0;
          load_mixed_pos(P, w, seg_begin, seg_pref, seg_shift, region, tb + tid, total, seg, p0);
          p0.base += copy_off;
          if (SHORT) {
            if (KIND == MIA_KIND_W) p0.loff = fmaf(-p0.zl, P.p_inv32, fmaf(-p0.zh, P.p_inv32, P.p_off32));
            p0.nh = make_float2(-p0.xh, -p0.yh);
            p0.nl = make_float2(-p0.xl, -p0.yl);
            p0.w2 = make_float2(p0.w, p0.w);
            if (KIND != MIA_KIND_W) p0.nz = make_float2(-p0.zh, -p0.zl);
          }
          // positions of the unit's region only (all but points on sub-box
          // faces): no per-pair slot check
          const bool all_in = __all_sync(0xffffffffu, !p0.valid || p0.slot >= 0);
          int i_lo = S, i_hi = 0;
          if (p0.valid) {
            if (FULL && P.full[2]) {
              i_lo = 0;
              i_hi = S;
            } else {
              // shapes are staged in line-of-sight order: only a window of them
              // can be within range of this position (conservative float bounds).
              // With a local neighbourhood the position sits in the cell's
              // periodic image, and its projected gap g to the cell bounds every
              // pair: g^2 beyond q_cut leaves nothing to bin, and for multipoles
              // |Pi| <= sqrt(q_cut - g^2) (plus 1e-4 q_cut under the root for
              // the FP32 rounding of the difference)
              float win = P.zwin;
              if (!FULL) {
                const float px = p0.xh + p0.xl, py = p0.yh + p0.yl;
                const float gx = fmaxf(0.0f, fmaxf(s_box[0] - px, px - s_box[1]));
                const float gy = fmaxf(0.0f, fmaxf(s_box[2] - py, py - s_box[3]));
                const float g2 = fmaf(gx, gx, gy * gy);
                if (g2 > P.q_cut) {
                  win = -1.0f;
                } else if (KIND == MIA_KIND_MULTIPOLES) {
                  win = fminf(win, sqrtf(fmaxf(P.q_cut - g2, 0.0f) + 1e-4f * P.q_cut) + P.zwin - P.range_los32);
                }
              }
              if (win >= 0.0f) {
                if (SHORT == 2) {  // (the line-of-sight reach spans the box: every staged shape)
                  i_lo = 0;
                  i_hi = S;
                } else {
                  z_window(Z, S, p0.zh + p0.zl, win, i_lo, i_hi);
                }
              }
            }
          }
          // the union over the warp is barely wider (neighbouring positions),
          // and every lane then reads the same staged shape in each iteration
          const int wlo = __reduce_min_sync(0xffffffffu, i_lo);
          const int whi = __reduce_max_sync(0xffffffffu, i_hi);
          if (p0.valid && wlo < whi) {
            if (all_in)
              shape_loop<KIND, FULL, VAR, 1, SHORT>(P, T, A, B, C, I, wlo, whi, p0, hv, w, o, sc, twoR, u.label,
                                                    my_binned);
            else
              shape_loop<KIND, FULL, VAR, 0, SHORT>(P, T, A, B, C, I, wlo, whi, p0, hv, w, o, sc, twoR, u.label,
                                                    my_binned);
          }
        }
      } else {
        int seg = 0;
        const double* D = reinterpret_cast<const double*>(smem + SL.shapes);
        const int M = P.shapes_per_unit;
        const float* Z = reinterpret_cast<const float*>(D + 7 * M);
        // warp-uniform iterations, so that a warp's lanes can agree on one shape range
        for (int tb = 0; tb < total; tb += blockDim.x) {
          const int t = tb + tid;
          int pidx = 0, code = 13;
          if (t < total) {
            while (t >= seg_pref[seg + 1]) ++seg;
            pidx = seg_begin[seg] + (t - seg_pref[seg]);
            code = seg_shift[seg];
          }
          const int plab = t < total ? w.plab_s[pidx] : region;
          const int slot = plab == region ? 0 : -1;
          const int base = 0;
          const double qx = w.px[pidx], qy = w.py[pidx], qz = w.pz[pidx], pw = w.pw[pidx];
          // the shapes that can bin with this position: the same conservative
          // FP32 window over the line-of-sight order as the mixed form (the
          // position's image next to the cell: code from the row's shift).
          // Every decision below stays the exact FP64 one.
          int i_lo = S, i_hi = 0;
          if (t < total) {
            if (FULL && P.full[2]) {
              i_lo = 0;
              i_hi = S;
            } else {
              float win = P.zwin;
              if (!FULL) {
                const float px = (float)(qx + (code % 3 - 1) * P.L), py = (float)(qy + ((code / 3) % 3 - 1) * P.L);
                const float gx = fmaxf(0.0f, fmaxf(s_box[0] - px, px - s_box[1]));
                const float gy = fmaxf(0.0f, fmaxf(s_box[2] - py, py - s_box[3]));
                const float g2 = fmaf(gx, gx, gy * gy);
                if (g2 > P.q_cut) {
                  win = -1.0f;
                } else if (KIND == MIA_KIND_MULTIPOLES) {
                  win = fminf(win, sqrtf(fmaxf(P.q_cut - g2, 0.0f) + 1e-4f * P.q_cut) + P.zwin - P.range_los32);
                }
              }
              if (win >= 0.0f) z_window(Z, S, (float)(qz + (code / 9 - 1) * P.L), win, i_lo, i_hi);
            }
          }
          const int wlo = __reduce_min_sync(0xffffffffu, i_lo);
          const int whi = __reduce_max_sync(0xffffffffu, i_hi);
          // one pair in the exact FP64 arithmetic, into the unit's histogram
          auto exact_pair = [&](int i, double x, double y, double z, double wp, int lab) {
            const PairResult r = pair_exact(P, T, D[i], D[M + i], D[2 * M + i], D[3 * M + i], D[4 * M + i],
                                            D[5 * M + i], x, y, z);
            if (r.bin < 0) return;
            const int sl = lab == region ? 0 : -1;
            const double ww = __dmul_rn(wp, D[6 * M + i]);
            const double sp = __dmul_rn(ww, r.ep);
            const double sx = __dmul_rn(ww, r.ex);
            double tv = 0.0;
            if (VAR) tv = __ddiv_rn(sp, twoR);
            const double vr = __dmul_rn(tv, tv);
            Fix128 fd, fp, fx, fv;
            bool ok = to_fix128(ww, sc.e128, fd);
            ok &= to_fix128(sp, sc.e128, fp);
            ok &= to_fix128(sx, sc.e128, fx);
            if (VAR) ok &= to_fix128(vr, sc.e128v, fv);
            if (sl >= 0 && ok) {
              const int hi = base + r.bin;
              atomicAdd(&h_cnt[hi], 1u);
              add_fix128(dd_q + 2 * hi, fd);
              add_fix128(sp_q + 2 * hi, fp);
              add_fix128(sx_q + 2 * hi, fx);
              if (VAR) add_fix128(vr_q + 2 * hi, fv);
            } else {
              acc_global(w, o, sc, nb, P.J, u.label, lab, r.bin, ww, sp, sx, vr, VAR);
              if (sl < 0) atomicOr(&w.status->flags, kStatusNoSlot);
              ++my_binned;
            }
          };
          // Two phases.  (1) Every lane tests its own pair with the shape of
          // the iteration: an FP32 range test from single floats, with a margin
          // for their rounding; the warp's survivors go to its ring as (shape,
          // lane).  (2) Whenever 32 are waiting, each lane takes one and runs
          // the exact FP64 arithmetic with the position of the lane that found
          // it.  A third of the candidates fail the range test; without the
          // ring the FP64 pipe would spend their share of every warp
          // instruction on idle lanes (1.35x on the 4M / 1M w step).  (The
          // mixed form does better without it: its binning is cheap enough
          // that the scattered shared-memory reads of phase (2) cost more than
          // the idle lanes.)
          (void)slot;
          const int lane = tid & 31;
          double2* WD = reinterpret_cast<double2*>(wpos) + 2 * (tid & ~31);
          int* WL = reinterpret_cast<int*>(reinterpret_cast<double2*>(wpos) + 2 * kThreads) + (tid & ~31);
          unsigned short* Q = ring + kRing * (tid >> 5);
          const bool valid = t < total;
          WD[2 * lane] = make_double2(qx, qy);
          WD[2 * lane + 1] = make_double2(qz, pw);
          WL[lane] = plab;
          __syncwarp();
          const float* XF = Z + M;
          const float* YF = Z + 2 * M;
          const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
          auto bin_entry = [&](unsigned e) {
            const int i = (int)(e >> 5), src = (int)(e & 31u);
            const double2 a = WD[2 * src], b = WD[2 * src + 1];
            exact_pair(i, a.x, a.y, b.x, b.y, WL[src]);
          };
          const unsigned below = (1u << lane) - 1u;
          unsigned head = 0, tail = 0;  // warp-uniform ring counters
          for (int i = wlo; i < whi; ++i) {
            const bool pass = valid && in_range_fp64<KIND>(P, XF[i], YF[i], Z[i], fx, fy, fz);
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (pass) Q[(tail + __popc(m & below)) & (kRing - 1)] = (unsigned short)((i << 5) | lane);
            tail += __popc(m);
            if (tail - head >= 32) {
              __syncwarp();
              const unsigned e = Q[(head + lane) & (kRing - 1)];
              head += 32;
              bin_entry(e);
              __syncwarp();
            }
          }
          __syncwarp();
          if ((unsigned)lane < tail - head) bin_entry(Q[(head + lane) & (kRing - 1)]);
          __syncwarp();
        }
      }
      __syncthreads();
    }

    // -- flush the unit's histogram
    const int a = u.label;
    const int b = region;
    const int copies = s_copies, stride = s_stride;
    for (int idx = tid; idx < nb; idx += blockDim.x) {
      const int bin = idx;
      unsigned cnt = 0;
      for (int c = 0; c < copies; ++c) cnt += h_cnt[c * stride + idx];
      if (cnt == 0) continue;
      my_binned += cnt;
      if (MIXED) {
        // the unit's exact partial of this (slot, bin): the high word plus the
        // copies' signed low words, added to the dataset's 64-bit sums
        // (integer adds: the totals do not depend on the order of the units)
        typedef unsigned long long u64;
        long long vdd = (long long)dd_hi[idx] << 32, vsp = (long long)sp_hi[idx] << 32,
                  vsx = (long long)sx_hi[idx] << 32, vvr = VAR ? (long long)vr_hi[idx] << 32 : 0;
        for (int c = 0; c < copies; ++c) {
          const int j = c * stride + idx;
          vdd += (long long)(int)dd_lo[j];
          vsp += (long long)(int)sp_lo[j];
          vsx += (long long)(int)sx_lo[j];
          if (VAR) vvr += (long long)(int)vr_lo[j];
        }
        atomicAdd(&o.npairs[bin], (u64)cnt);
        atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[bin]), (u64)vdd);
        atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[bin]), (u64)vsp);
        atomicAdd(reinterpret_cast<u64*>(&w.acc_sx[bin]), (u64)vsx);
        if (VAR) atomicAdd(reinterpret_cast<u64*>(&w.acc_vr[bin]), (u64)vvr);
        if (P.J > 0) {
          const size_t ia = (size_t)(1 + a) * nb + bin;
          atomicAdd(&o.npairs[ia], (u64)cnt);
          atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[ia]), (u64)vdd);
          atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[ia]), (u64)vsp);
          if (b != a) {
            const size_t ibb = (size_t)(1 + b) * nb + bin;
            atomicAdd(&o.npairs[ibb], (u64)cnt);
            atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[ibb]), (u64)vdd);
            atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[ibb]), (u64)vsp);
          }
        }
      } else {
        // the unit's exact 128-bit partials into the dataset's sums
        typedef unsigned long long u64;
        const Fix128 vd{dd_q[2 * idx], dd_q[2 * idx + 1]}, vp{sp_q[2 * idx], sp_q[2 * idx + 1]},
            vx{sx_q[2 * idx], sx_q[2 * idx + 1]};
        u64* const add = reinterpret_cast<u64*>(w.acc_dd);
        u64* const asp = reinterpret_cast<u64*>(w.acc_sp);
        atomicAdd(&o.npairs[bin], (u64)cnt);
        add_fix128(add + 2 * bin, vd);
        add_fix128(asp + 2 * bin, vp);
        add_fix128(reinterpret_cast<u64*>(w.acc_sx) + 2 * bin, vx);
        if (VAR) add_fix128(reinterpret_cast<u64*>(w.acc_vr) + 2 * bin, Fix128{vr_q[2 * idx], vr_q[2 * idx + 1]});
        if (P.J > 0) {
          const size_t ia = (size_t)(1 + a) * nb + bin;
          atomicAdd(&o.npairs[ia], (u64)cnt);
          add_fix128(add + 2 * ia, vd);
          add_fix128(asp + 2 * ia, vp);
          if (b != a) {
            const size_t ibb = (size_t)(1 + b) * nb + bin;
            atomicAdd(&o.npairs[ibb], (u64)cnt);
            add_fix128(add + 2 * ibb, vd);
            add_fix128(asp + 2 * ibb, vp);
          }
        }
      }
    }
    // binned-pair total of the dataset, for the throughput figure
    for (int of = 16; of > 0; of >>= 1) my_binned += __shfl_down_sync(0xffffffffu, my_binned, of);
    if ((tid & 31) == 0 && my_binned) atomicAdd(&w.status->binned, my_binned);
    __syncthreads();
  }
}

// FP64 re-test of the pairs the mixed kernel could not decide in FP32; their
// FP64 terms join the dataset's fixed-point sums at the same scales.  Every
// re-tested pair adds to one of the nb all-pairs sums, so a block first sums
// those in shared memory (64-bit integer atomics, flushed once per block);
// the per-region sums, spread over (1 + J) nb words, go to global memory
// directly.  (With 2.4M pairs on a few hundred words, global atomics alone
// serialised on their L2 lines.)
__global__ void k_edge_retest(Params P, Work w, Out o, int agg) {
  extern __shared__ __align__(8) unsigned long long rt_smem[];
  if (w.status->flags & kStatusRange) return;  // the measurement ends in MIA_ERR_RANGE
  typedef unsigned long long u64;
  const int nb = P.nb;
  const int want_var = P.want_variance;
  u64* s_cnt = rt_smem;          // nb each: count, w, S+D, SxD (, variance terms)
  u64* s_dd = s_cnt + nb;
  u64* s_sp = s_dd + nb;
  u64* s_sx = s_sp + nb;
  u64* s_vr = s_sx + nb;
  const int words = agg ? (4 + want_var) * nb : 0;  // (agg = 0: too many bins for shared memory)
  for (int i = threadIdx.x; i < words; i += blockDim.x) rt_smem[i] = 0ull;
  __syncthreads();
  const unsigned long long n_raw = w.status->edge_count;
  const unsigned long long n = n_raw < (unsigned long long)w.edge_capacity ? n_raw : (unsigned long long)w.edge_capacity;
  const double twoR = dataset_twoR(w.reg, P.J);
  const Scales sc = dataset_scales(w.status, twoR);
  unsigned long long binned = 0;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const int2 e = w.edges[k];
    const int si = e.x, pi = e.y;
    PairResult r = pair_exact(P, *w.tables, w.sx[si], w.sy[si], w.sz[si], w.sax[si], w.say[si], w.se[si], w.px[pi],
                              w.py[pi], w.pz[pi]);
    if (r.bin < 0) continue;
    const double ww = __dmul_rn(w.pw[pi], w.sws[si]);
    const double sp = __dmul_rn(ww, r.ep);
    const double sx = __dmul_rn(ww, r.ex);
    const double tv = __ddiv_rn(sp, twoR);
    const long long vd = __double2ll_rn(ww * sc.sd_dd), vp = __double2ll_rn(sp * sc.sd_sp),
                    vx = __double2ll_rn(sx * sc.sd_sp), vv = want_var ? __double2ll_rn(tv * tv * sc.sd_vr) : 0;
    const int bin = r.bin;
    if (agg) {
      atomicAdd(&s_cnt[bin], 1ull);
      atomicAdd(&s_dd[bin], (u64)vd);
      atomicAdd(&s_sp[bin], (u64)vp);
      atomicAdd(&s_sx[bin], (u64)vx);
      if (want_var) atomicAdd(&s_vr[bin], (u64)vv);
    } else {
      atomicAdd(&o.npairs[bin], 1ULL);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[bin]), (u64)vd);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[bin]), (u64)vp);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_sx[bin]), (u64)vx);
      if (want_var) atomicAdd(reinterpret_cast<u64*>(&w.acc_vr[bin]), (u64)vv);
    }
    if (P.J > 0) {
      const int a = w.slab_s[si], b = w.plab_s[pi];
      const size_t ia = (size_t)(1 + a) * nb + bin;
      atomicAdd(&o.npairs[ia], 1ULL);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[ia]), (u64)vd);
      atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[ia]), (u64)vp);
      if (b != a) {
        const size_t ib = (size_t)(1 + b) * nb + bin;
        atomicAdd(&o.npairs[ib], 1ULL);
        atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[ib]), (u64)vd);
        atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[ib]), (u64)vp);
      }
    }
    ++binned;
  }
  for (int of = 16; of > 0; of >>= 1) binned += __shfl_down_sync(0xffffffffu, binned, of);
  if ((threadIdx.x & 31) == 0 && binned) atomicAdd(&w.status->binned, binned);
  __syncthreads();
  for (int bin = threadIdx.x; agg && bin < nb; bin += blockDim.x) {
    const u64 c = s_cnt[bin];
    if (!c) continue;
    atomicAdd(&o.npairs[bin], c);
    atomicAdd(reinterpret_cast<u64*>(&w.acc_dd[bin]), s_dd[bin]);
    atomicAdd(reinterpret_cast<u64*>(&w.acc_sp[bin]), s_sp[bin]);
    atomicAdd(reinterpret_cast<u64*>(&w.acc_sx[bin]), s_sx[bin]);
    if (want_var) atomicAdd(reinterpret_cast<u64*>(&w.acc_vr[bin]), s_vr[bin]);
  }
}

// The dataset's exact fixed-point sums into the output doubles (w and S+D per
// region, SxD and the variance terms), before post-processing.  Mixed form:
// 64-bit sums.  FP64 form: 128-bit sums, added to what the output doubles
// already hold (the terms that were not finite, else zero).
__global__ void k_fixed_out(Params P, Work w, Out o) {
  const Scales sc = dataset_scales(w.status, dataset_twoR(w.reg, P.J));
  const int n1 = (1 + P.J) * P.nb;
  typedef unsigned long long u64;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1; i += gridDim.x * blockDim.x) {
    if (P.precision == MIA_MIXED) {
      o.dd[i] = (double)w.acc_dd[i] * sc.inv_dd;
      o.splus[i] = (double)w.acc_sp[i] * sc.inv_sp;
      if (i < P.nb) {
        o.scross[i] = (double)w.acc_sx[i] * sc.inv_sp;
        if (P.want_variance) o.variance[i] = (double)w.acc_vr[i] * sc.inv_vr;
      }
    } else {
      auto val = [&](const long long* a, double inv) {
        const u64* q = reinterpret_cast<const u64*>(a) + 2 * (size_t)i;
        return fix128_value(q[0], q[1], inv);
      };
      o.dd[i] = __dadd_rn(val(w.acc_dd, sc.inv128), o.dd[i]);
      o.splus[i] = __dadd_rn(val(w.acc_sp, sc.inv128), o.splus[i]);
      if (i < P.nb) {
        o.scross[i] = __dadd_rn(val(w.acc_sx, sc.inv128), o.scross[i]);
        if (P.want_variance) o.variance[i] = __dadd_rn(val(w.acc_vr, sc.inv128v), o.variance[i]);
      }
    }
  }
}

// Histogram words per array for the mixed form: nb bins at least, and as
// much more (for private copies, up to 32) as fits without lowering the
// blocks per SM that the registers allow.
template <int MIXED, int VAR, int KIND, int FULL>
cudaError_t hist_words_for(const Params& P, int& hw) {
  hw = P.nb;
  if (!MIXED) return cudaSuccess;
  auto kern = k_pairs<MIXED, VAR, KIND, FULL, 0>;
  int dev = 0, smem_sm = 0, smem_blk = 0, reserved = 0, b_reg = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b_reg, kern, kThreads, 0);
  cudaFuncAttributes fa;
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
#ifdef MIA_MAX_BLOCKS_PER_SM
  if (b_reg > MIA_MAX_BLOCKS_PER_SM) b_reg = MIA_MAX_BLOCKS_PER_SM;
#endif
  if (b_reg < 1) return cudaSuccess;
  long long room = (long long)smem_sm / b_reg - reserved - (long long)fa.sharedSizeBytes;
  if (room > smem_blk - (long long)fa.sharedSizeBytes) room = smem_blk - (long long)fa.sharedSizeBytes;
  const int hw_max = 32 * (P.nb | 1);
  int best = hw;
  for (int c = hw_max; c > hw; c -= 16)
    if ((long long)smem_layout(P.shapes_per_unit, c, P.nb, MIXED, VAR).total <= room) {
      best = c;
      break;
    }
  hw = best;
  return cudaSuccess;
}

// The short pair path: histogram arrays of kHistShort (kHistShortVar) words,
// as many copies as they hold, and the blocks per SM that this leaves.
template <int KIND, int SHORT, int VAR>
cudaError_t launch_short(const Params& P, const Dataset* ds, int n_ds, const unsigned long long* wu_prefix,
                         unsigned long long* wu_next, cudaStream_t st, int num_sms) {
  auto kern = k_pairs<1, VAR, KIND, 0, SHORT>;
  constexpr int KS = VAR ? kHistShortVar : kHistShort;
  const size_t smem = smem_layout(P.shapes_per_unit, KS, P.nb, 1, VAR).total;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (e != cudaSuccess) return e;
#ifdef MIA_MAX_BLOCKS_PER_SM
  if (per_sm > MIA_MAX_BLOCKS_PER_SM) per_sm = MIA_MAX_BLOCKS_PER_SM;
#endif
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kern<<<num_sms * per_sm, kThreads, smem, st>>>(P, ds, n_ds, wu_prefix, wu_next, KS);
  return cudaGetLastError();
}

template <int MIXED, int VAR, int KIND, int FULL>
cudaError_t launch_one(const Params& P, const Dataset* ds, int n_ds, const unsigned long long* wu_prefix,
                       unsigned long long* wu_next, cudaStream_t st, int num_sms) {
  int hw = 0;
  cudaError_t e = hist_words_for<MIXED, VAR, KIND, FULL>(P, hw);
  if (e != cudaSuccess) return e;
  auto kern = k_pairs<MIXED, VAR, KIND, FULL, 0>;
  const int hw0 = P.nb;
  int per_sm = 0, per_sm0 = 0;
  size_t smem = smem_layout(P.shapes_per_unit, hw0, hw0, MIXED, VAR).total;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm0, kern, kThreads, smem);
  if (e != cudaSuccess) return e;
#ifdef MIA_MAX_BLOCKS_PER_SM
  if (per_sm0 > MIA_MAX_BLOCKS_PER_SM) per_sm0 = MIA_MAX_BLOCKS_PER_SM;
#endif
  per_sm = per_sm0;
  // the copies must not cost a block per SM
  while (hw > hw0) {
    const size_t s1 = smem_layout(P.shapes_per_unit, hw, hw0, MIXED, VAR).total;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1);
    if (e != cudaSuccess) return e;
    int b = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kThreads, s1);
    if (e != cudaSuccess) return e;
    if (b >= per_sm0) {
      smem = s1;
      per_sm = per_sm0;
      break;
    }
    hw = hw - 16 > hw0 ? hw - 16 : hw0;
  }
  if (hw == hw0) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kern<<<num_sms * per_sm, kThreads, smem, st>>>(P, ds, n_ds, wu_prefix, wu_next, hw);
  return cudaGetLastError();
}

template <int MIXED, int VAR>
cudaError_t launch_kind(const Params& P, const Dataset* ds, int n_ds, const unsigned long long* wu_prefix,
                        unsigned long long* wu_next, cudaStream_t st, int num_sms) {
  const bool full = P.full[0] || P.full[1] || P.full[2];
  // the short path: local neighbourhoods, or (w) a line-of-sight reach that
  // spans the box with the plane local
  if (MIXED && P.short_ok && (P.nb | 1) <= (VAR ? kHistShortVar : kHistShort)) {
    if (!full)
      return P.kind == MIA_KIND_W ? launch_short<MIA_KIND_W, 1, VAR>(P, ds, n_ds, wu_prefix, wu_next, st, num_sms)
                                  : launch_short<MIA_KIND_MULTIPOLES, 1, VAR>(P, ds, n_ds, wu_prefix, wu_next, st,
                                                                             num_sms);
    if (P.short_wrap) return launch_short<MIA_KIND_W, 2, VAR>(P, ds, n_ds, wu_prefix, wu_next, st, num_sms);
  }
  if (P.kind == MIA_KIND_W)
    return full ? launch_one<MIXED, VAR, MIA_KIND_W, 1>(P, ds, n_ds, wu_prefix, wu_next, st, num_sms)
                : launch_one<MIXED, VAR, MIA_KIND_W, 0>(P, ds, n_ds, wu_prefix, wu_next, st, num_sms);
  return full ? launch_one<MIXED, VAR, MIA_KIND_MULTIPOLES, 1>(P, ds, n_ds, wu_prefix, wu_next, st, num_sms)
              : launch_one<MIXED, VAR, MIA_KIND_MULTIPOLES, 0>(P, ds, n_ds, wu_prefix, wu_next, st, num_sms);
}

// Global work-unit index of each dataset's first unit: a dataset has n_wu
// runs times reg_slots region slots.
__global__ void k_batch_prefix(const Dataset* ds, int n, int reg_slots, unsigned long long* prefix) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int i = 0; i < n; ++i) {
      prefix[i] = acc;
      acc += ds[i].w.status->n_wu * (unsigned long long)reg_slots;
    }
    prefix[n] = acc;
  }
}

}  // namespace

cudaError_t launch_batch_prefix(const Dataset* ds_dev, int n_ds, int reg_slots, unsigned long long* wu_prefix,
                                cudaStream_t st) {
  k_batch_prefix<<<1, 32, 0, st>>>(ds_dev, n_ds, reg_slots, wu_prefix);
  return cudaGetLastError();
}

cudaError_t launch_fixed_out(const Params& P, const Work& w, const Out& o, cudaStream_t st) {
  const int n1 = (1 + P.J) * P.nb;
  const int blocks = (n1 + 255) / 256;
  k_fixed_out<<<blocks < 1024 ? blocks : 1024, 256, 0, st>>>(P, w, o);
  return cudaGetLastError();
}

cudaError_t launch_edge_retest(const Params& P, const Work& w, const Out& o, cudaStream_t st, int num_sms) {
  // the all-pairs sums in shared memory when they fit in 48 KB (nb <= 1228)
  size_t smem = sizeof(unsigned long long) * (size_t)(4 + (P.want_variance ? 1 : 0)) * P.nb;
  const int agg = smem <= 48 * 1024 ? 1 : 0;
  if (!agg) smem = 0;
  k_edge_retest<<<num_sms * 4, 256, smem, st>>>(P, w, o, agg);
  return cudaGetLastError();
}

cudaError_t launch_pairs(const Params& P, const Dataset* ds_dev, int n_ds, const unsigned long long* wu_prefix,
                         unsigned long long* wu_next, cudaStream_t st, int num_sms) {
  if (P.precision == MIA_MIXED)
    return P.want_variance ? launch_kind<1, 1>(P, ds_dev, n_ds, wu_prefix, wu_next, st, num_sms)
                           : launch_kind<1, 0>(P, ds_dev, n_ds, wu_prefix, wu_next, st, num_sms);
  return P.want_variance ? launch_kind<0, 1>(P, ds_dev, n_ds, wu_prefix, wu_next, st, num_sms)
                         : launch_kind<0, 0>(P, ds_dev, n_ds, wu_prefix, wu_next, st, num_sms);
}

}  // namespace mia
