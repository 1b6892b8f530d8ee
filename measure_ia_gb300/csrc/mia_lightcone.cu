// Lightcone pair counts: the brute-force counters of MeasureIALightcone
// (measure_w_lightcone.py:45-343, measure_m_lightcone.py:45-363) with the
// per-patch re-counts of the pooled jackknife driver
// (measure_jackknife.py:265-484) folded into one pass.
//
// The reference loops over positions and, for each, evaluates every shape
// with numpy.  Here the shapes are counting-sorted into a grid of
// (DEC band, comoving-distance slab, RA bin) cells; the positions, sorted into
// the same grid, are taken one per warp by a persistent kernel, and each warp
// reads only the cells its position's separation window can reach.  The
// window is a superset: every candidate is decided by the reference's own
// FP64 operation sequence (division-free FP64 bound first, then the exact
// arithmetic with _rn intrinsics), so the bins are the reference's bit for bit.
//
// Jackknife: the realisation without patch i holds the pairs with neither
// member in i.  With A[i] = sums over pairs whose position is in i and B[i] =
// sums over pairs whose shape is in i but whose position is not, realisation
// i = total - A[i] - B[i].  A is accumulated per warp in shared memory (the
// positions are grid-sorted, so a warp's patch changes rarely); B, the pairs
// that straddle two patches, goes to global atomics.
//
// Every sum is an exact fixed-point integer (scale 2^E with the largest
// possible term at 2^46, so a term keeps every bit down to 2^-46 of the
// largest one): a warp's partials are 64-bit and flushed before 2^16 terms
// can reach one, the totals 128-bit (Fix128).  The sums do not depend on the
// order in which warps meet the pairs, and total - A[i] - B[i] is exact.
#include <cstdio>
#include <cstdlib>

#include "mia_internal.cuh"

namespace mia {

namespace {

constexpr int kLcMaxWarps = 8;
constexpr int kLcChunk = 4;            // positions per warp grab
constexpr double kDegToRad = 3.141592653589793 / 180.0;

struct LcGrid {
  double ra0, inv_ra, dec0, inv_dec, chi0, inv_chi;
  int n_ra, n_dec, n_chi;
};

__device__ __forceinline__ int cell_1d(double x, double x0, double inv, int n) {
  const double t = (x - x0) * inv;     // monotone in x: window bounds and objects agree
  if (!(t >= 0.0)) return 0;
  if (t >= (double)n) return n - 1;
  return (int)t;
}

__device__ __forceinline__ int cell_of(const LcGrid& g, double ra, double dec, double chi) {
  const int a = cell_1d(ra, g.ra0, g.inv_ra, g.n_ra);
  const int d = cell_1d(dec, g.dec0, g.inv_dec, g.n_dec);
  const int c = cell_1d(chi, g.chi0, g.inv_chi, g.n_chi);
  return (d * g.n_chi + c) * g.n_ra + a;
}

__global__ void k_lc_cells(const double* __restrict__ ra, const double* __restrict__ dec,
                           const double* __restrict__ chi, long long n, LcGrid g, int* __restrict__ cell,
                           int* __restrict__ count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c = cell_of(g, ra[i], dec[i], chi[i]);
    cell[i] = c;
    atomicAdd(&count[c], 1);
  }
}

struct LcSorted {   // one sample in cell order
  double *ra, *dec, *chi, *w, *aux0, *aux1, *aux2;   // positions: cos_dec, cx, cy; shapes: e, c2a, s2a
  int* patch;
  float4* hl;          // (ra_hi, ra_lo, dec_hi, dec_lo): x = hi + lo to ~2^-48 relative
  float2* chl;         // (chi_hi, chi_lo)
};

__device__ __forceinline__ float2 split(double x) {
  const float hi = __double2float_rn(x);
  return make_float2(hi, __double2float_rn(x - (double)hi));
}

// (also the sample's largest |w| -- for shapes max(|w|, |w e|) -- as a bit
// pattern into wmax: non-negative doubles order as their integer patterns)
__global__ void k_lc_scatter(mia_lc_sample in, long long n, const int* __restrict__ cell, int* __restrict__ fill,
                             LcSorted out, int is_pos, int with_shapes, unsigned long long* __restrict__ wmax) {
  unsigned long long mx = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double wa = fabs(in.w[i]);
    const double mw = (!is_pos && with_shapes) ? fmax(wa, fabs(in.w[i] * in.e[i])) : wa;
    const unsigned long long bits = (unsigned long long)__double_as_longlong(mw);
    mx = bits > mx ? bits : mx;
    const int d = atomicAdd(&fill[cell[i]], 1);
    const double ra = in.ra[i], dec = in.dec[i], chi = in.chi[i];
    out.ra[d] = ra;
    out.dec[d] = dec;
    out.chi[d] = chi;
    out.w[d] = in.w[i];
    out.patch[d] = in.patch ? in.patch[i] : 0;
    const float2 a = split(ra), b = split(dec);
    out.hl[d] = make_float4(a.x, a.y, b.x, b.y);
    out.chl[d] = split(chi);
    if (is_pos) {
      const double c = in.cos_dec[i];
      out.aux0[d] = c;
      out.aux1[d] = kDegToRad * chi * c;   // dx ~ (ra_s - ra_p) * cx, few ulp from the reference's dx
      out.aux2[d] = kDegToRad * chi;       // dy ~ (dec_s - dec_p) * cy
    } else if (with_shapes) {
      // w_s |e| cos 2phi_a and w_s |e| sin 2phi_a: a pair's S+D and SxD terms are
      // then -w_p (wa cos 2phi_s + wb sin 2phi_s) and -w_p (wb cos 2phi_s - wa sin 2phi_s)
      const double we = in.w[i] * in.e[i];
      out.aux0[d] = in.e[i];
      out.aux1[d] = we * in.c2a[i];
      out.aux2[d] = we * in.s2a[i];
    }
  }
  for (int of = 16; of > 0; of >>= 1) {
    const unsigned long long o = __shfl_down_sync(0xffffffffu, mx, of);
    mx = o > mx ? o : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(wmax, mx);
}

struct LcParams {
  int n_r, n_p, nb, n_patch, Q;
  int n_qbreak, n_pbreak;
  double h_extra, h2, rp_cut, r_lim, pi_lo, pi_hi;
  float qf_hi;                 // FP32 prefilter bound on q (r_lim^2 (1 + 1e-4))
  float los_lo, los_hi;        // w: FP32 prefilter bounds on Pi
  float qa, qb, pa, pb;        // first guesses of the table interval: log2(q) * qa + qb, x * pa + pb
  int unit;                    // unit weights: DD is the pair count, not summed
  int hq;                      // value arrays in a warp's histogram: Q, or 0 (unit-weight counts)
  int flush_steps;             // half-steps between flushes of the warp partials (2..kLcFlushSteps)
  LcGrid g;
  long long n_pos;
};

// Per-position window and FP32 constants, computed once per position
// (k_lc_windows) instead of once per warp in the pair kernel.
struct LcWin {
  int d0, d1, a0, a1, c0, c1;
  float kx, ky;                // Mpc per degree of RA / DEC difference (times h_extra for w)
  float gq, gqp, gmu, gl;      // absolute error bounds (see k_lc_windows)
  // the position and the window's half-widths in RA / DEC cell units, for
  // trimming each DEC row's RA range to the window's ellipse (sra < 0: no trim);
  // multipoles also in distance-slab units (schi > 0): r^2 = r_p^2 + Pi^2, so
  // a slab's distance gap narrows the ellipse too
  float tra, tdec, sra, sdec, tchi, schi;
};

// Per sorted position: the cell ranges its separation window reaches (a
// superset; the pair tests decide) and the FP32 constants of the prefilter.
// Error bounds: each hi/lo coordinate is within 2^-48 of itself, so a
// difference of two is within 2^-47 of the larger, which the window bounds;
// ep bounds that error on the projected terms ax, ay (Mpc), gl on the
// line-of-sight difference lf.  The FP32 arithmetic itself stays within
// 1.2e-6 relative of q (the guard, kRelGuard, is 4e-6).
template <int KIND>
__global__ void k_lc_windows(const LcParams P, const LcSorted pos, LcWin* __restrict__ win) {
  const LcGrid& g = P.g;
  const double hx = KIND == MIA_KIND_W ? P.h_extra : 1.0;
  for (long long ip = blockIdx.x * (long long)blockDim.x + threadIdx.x; ip < P.n_pos;
       ip += (long long)gridDim.x * blockDim.x) {
    const double ra_n = pos.ra[ip], dec_n = pos.dec[ip], chi_n = pos.chi[ip], cos_n = pos.aux0[ip];
    const double den = fabs(hx * chi_n);
    const double span_dec = den > 1e-300 ? P.r_lim / den / kDegToRad * (1.0 + 1e-6) + 1e-9 : 1e300;
    const double den_ra = den * fabs(cos_n);
    const double span_ra = den_ra > 1e-300 ? P.r_lim / den_ra / kDegToRad * (1.0 + 1e-6) + 1e-9 : 1e300;
    const double m = 1e-9 * (fabs(chi_n) + P.r_lim + fabs(P.pi_lo) + fabs(P.pi_hi)) + 1e-9;
    double chi_lo, chi_hi;
    if (KIND == MIA_KIND_W) {
      chi_lo = chi_n + P.pi_lo - m;
      chi_hi = chi_n + P.pi_hi + m;
    } else {
      chi_lo = chi_n - P.r_lim - m;
      chi_hi = chi_n + P.r_lim + m;
    }
    LcWin w;
    w.d0 = cell_1d(dec_n - span_dec, g.dec0, g.inv_dec, g.n_dec);
    w.d1 = cell_1d(dec_n + span_dec, g.dec0, g.inv_dec, g.n_dec);
    w.a0 = cell_1d(ra_n - span_ra, g.ra0, g.inv_ra, g.n_ra);
    w.a1 = cell_1d(ra_n + span_ra, g.ra0, g.inv_ra, g.n_ra);
    w.c0 = cell_1d(chi_lo, g.chi0, g.inv_chi, g.n_chi);
    w.c1 = cell_1d(chi_hi, g.chi0, g.inv_chi, g.n_chi);
    const double kxd = kDegToRad * chi_n * cos_n * hx, kyd = kDegToRad * chi_n * hx;
    w.kx = (float)kxd;
    w.ky = (float)kyd;
    const double ep = 1.1 * 7.2e-15 * ((fabs(ra_n) + fmin(span_ra, 1e30)) * fabs(kxd) +
                                       (fabs(dec_n) + fmin(span_dec, 1e30)) * fabs(kyd));
    const double gld = 1.1 * 7.2e-15 * (2.0 * fabs(chi_n) + P.r_lim + fabs(P.pi_lo) + fabs(P.pi_hi));
    w.gl = (float)gld;
    // on q (w: r_p^2; multipoles: r^2, which adds the lf term) with sqrt(q) <= 1.0001 r_lim
    w.gq = (float)(2.1 * P.r_lim * (ep + (KIND == MIA_KIND_W ? 0.0 : gld)) + ep * ep + gld * gld);
    w.gqp = (float)(P.h2 * (2.1 * P.r_lim * ep + ep * ep));   // on r_p^2 (the multipoles' cut)
    w.gmu = (float)(2.0 * (gld + ep));                          // times 1/r, on mu
    w.tra = (float)((ra_n - g.ra0) * g.inv_ra);
    w.tdec = (float)((dec_n - g.dec0) * g.inv_dec);
    const double sra = span_ra * g.inv_ra, sdec = span_dec * g.inv_dec;
    const bool trim = sra < 1e6 && sdec < 1e6 && sdec > 1e-6 && fabs((double)w.tra) < 1e6 && fabs((double)w.tdec) < 1e6;
    w.sra = trim ? (float)sra : -1.0f;
    w.sdec = trim ? (float)sdec : 1.0f;
    w.tchi = (float)((chi_n - g.chi0) * g.inv_chi);
    const double schi = (P.r_lim * (1.0 + 1e-6) + m) * g.inv_chi;
    w.schi = (KIND == MIA_KIND_MULTIPOLES && trim && schi > 1e-6 && schi < 1e6 && fabs((double)w.tchi) < 1e6)
                 ? (float)schi : -1.0f;
    win[ip] = w;
  }
}

struct LcAcc {
  unsigned long long* A128;    // [max(1, n_patch)][Q][nb] Fix128 (lo, hi)
  unsigned long long* B128;    // [n_patch][Q][nb] Fix128
  double* A;                   // [max(1, n_patch)][Q][nb]: terms that are not finite (else 0)
  double* B;                   // [n_patch][Q][nb]: the same
  const unsigned long long* wmax;   // largest |w| of the positions, max(|w|, |w e|) of the shapes
  unsigned long long* cA;      // [max(1, n_patch)][nb]
  unsigned long long* cB;      // [n_patch][nb]
  unsigned* next;              // work counter
  unsigned* status;
};

// Fixed-point exponent of a counter from the largest possible term m (weight
// products; the shape terms are bounded by |w_p| |w_s e|): 64-bit warp
// partials, m 2^E <= 2^46, so that 2^16 terms fit one; wide (128-bit)
// partials, m 2^E <= 2^88 (fix128_exponent).
__device__ inline int lc_exponent(const unsigned long long* wmax, int wide) {
  double m = __longlong_as_double((long long)wmax[0]) * __longlong_as_double((long long)wmax[1]);
  if (!(m > 0.0) || !(m < 1e300)) m = 1.0;
  if (wide) return fix128_exponent(m);
  const int e = ilogb(70368744177664.0 / m);  // 2^46
  return e > 1000 ? 1000 : (e < -1000 ? -1000 : e);
}
constexpr int kLcFlushSteps = 2000;   // half-steps (<= 32 terms each) between partial flushes (at most)

// shared-memory bytes of the tables: double and FP32 breaks, bins; 16-byte rounded
constexpr size_t kLcTableBytes = (2 * MIA_MAX_BREAKS * 8 + 2 * MIA_MAX_BREAKS * 4 + 2 * (MIA_MAX_BREAKS + 1) * 4 + 15) & ~size_t(15);

struct LcTables {              // bin tables, passed by value (2.3 KB of launch parameters)
  double qbr[MIA_MAX_BREAKS], pbr[MIA_MAX_BREAKS];
  int qbn[MIA_MAX_BREAKS + 1], pbn[MIA_MAX_BREAKS + 1];
};

// searchsorted(breaks, x, side='right') -> bins[]
__device__ __forceinline__ int lookup(const double* br, const int* bins, int n, double x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (br[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return bins[lo];
}

// Interval of an approximate x in FP32 among the (FP32-rounded) breaks: from
// a first guess t0, walk to t = #{breaks <= x}, the binary search's answer.
// `near` is set when a break lies within tol of x, where x could be on the
// wrong side of it.
__device__ __forceinline__ int lookup_f(const float* br, const int* bins, int n, float x, float t0, float tol,
                                        bool& near) {
  int t = (int)fminf(fmaxf(t0, 0.0f), (float)n);
  while (t < n && br[t] <= x) ++t;
  while (t > 0 && br[t - 1] > x) --t;
  if (t > 0 && x - br[t - 1] <= tol) near = true;
  if (t < n && br[t] - x <= tol) near = true;
  return bins[t];
}

// FP32 decisions: the separation terms from the hi/lo coordinates are within
// ~1e-6 relative of the reference's (plus an absolute term from the 2^-48
// hi/lo representation, bounded per position); pairs within kRelGuard of a
// breakpoint (or of the r_p cut) take the reference's exact FP64 sequence.
constexpr float kRelGuard = 4e-6f;
constexpr int kQueue = 64;         // per-warp queue of survivors (int4 entries)

// UNIT: every weight is 1 (DD is the pair count; no weight products summed).
// WIDE: 128-bit warp partials (two words per sum) instead of 64-bit ones.
template <int KIND, int SHAPES, int JK, int UNIT, int WIDE>
__global__ void __launch_bounds__(kLcMaxWarps * 32, 4)
k_lc_pairs(const LcParams P, const LcTables T, const LcSorted pos, const LcSorted shp, const int* __restrict__ start,
           const LcWin* __restrict__ win, const LcAcc acc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  const int nb = P.nb;
  constexpr int Q = SHAPES ? 3 : 1;
  // tables (double and FP32 breaks), per-warp queues, then per-warp histograms
  double* s_qbr = reinterpret_cast<double*>(smem_raw);
  double* s_pbr = s_qbr + MIA_MAX_BREAKS;
  float* s_qbf = reinterpret_cast<float*>(s_pbr + MIA_MAX_BREAKS);
  float* s_pbf = s_qbf + MIA_MAX_BREAKS;
  int* s_qbn = reinterpret_cast<int*>(s_pbf + MIA_MAX_BREAKS);
  int* s_pbn = s_qbn + (MIA_MAX_BREAKS + 1);
  int4* queues = reinterpret_cast<int4*>(smem_raw + kLcTableBytes);
  int4* queue = queues + warp * kQueue;
  // per warp: hq * nb signed 64-bit partial sums, then nb u32 counts
  unsigned long long* hist_base = reinterpret_cast<unsigned long long*>(queues + n_warps * kQueue);
  constexpr int PW = WIDE ? 2 : 1;   // 64-bit words per partial sum
  const int hw = PW * P.hq * nb;
  unsigned long long* h = hist_base + (size_t)warp * ((size_t)hw + (nb + 1) / 2);
  unsigned* hc = reinterpret_cast<unsigned*>(h + hw);
  const int E = lc_exponent(acc.wmax, WIDE);
  int steps = 0;   // half-steps (<= 32 terms each) since the last flush (warp-uniform)
  for (int i = threadIdx.x; i < MIA_MAX_BREAKS; i += blockDim.x) {
    s_qbr[i] = T.qbr[i];
    s_pbr[i] = T.pbr[i];
    s_qbf[i] = __double2float_rn(T.qbr[i]);
    s_pbf[i] = __double2float_rn(T.pbr[i]);
  }
  for (int i = threadIdx.x; i <= MIA_MAX_BREAKS; i += blockDim.x) {
    s_qbn[i] = T.qbn[i];
    s_pbn[i] = T.pbn[i];
  }
  for (int i = lane; i < hw; i += 32) h[i] = 0ull;
  for (int i = lane; i < nb; i += 32) hc[i] = 0u;
  __syncthreads();

  int cur = -1;  // patch whose sums the warp's histogram holds
  int cnt = 0;   // entries in the warp's queue

  auto flush_hist = [&](int p) {
    __syncwarp();
    if (p >= 0) {
      unsigned long long* dst = acc.A128 + (size_t)p * Q * nb * 2;
      unsigned long long* cdst = acc.cA + (size_t)p * nb;
      for (int i = lane; i < P.hq * nb; i += 32) {
        Fix128 v;
        if (WIDE) {
          v = Fix128{h[2 * i], h[2 * i + 1]};
          h[2 * i] = 0ull;
          h[2 * i + 1] = 0ull;
        } else {
          v = Fix128{h[i], (unsigned long long)((long long)h[i] >> 63)};   // sign-extended
          h[i] = 0ull;
        }
        if (v.lo | v.hi) add_fix128(dst + 2 * i, v);
      }
      for (int i = lane; i < nb; i += 32) {
        const unsigned c = hc[i];
        if (c) atomicAdd(&cdst[i], (unsigned long long)c);
        hc[i] = 0u;
      }
    }
    __syncwarp();
  };

  // a pair's terms into the warp's histogram (A, patch cur) and, when the
  // shape lies in another patch, into B; a term that is not finite goes to
  // the double arrays instead (a bin holding one reads inf or NaN)
  auto accumulate = [&](int j, int bin, double ww, double sp, double sx) {
    Fix128 f[3];
    bool ok[3] = {true, true, true};
    const double v[3] = {ww, sp, sx};
    const int q0 = UNIT ? 1 : 0, q1 = SHAPES ? 3 : 1;
    for (int q = q0; q < q1; ++q) {
      // a finite term within the partials' range (64-bit: |t| 2^E < 2^47,
      // which the bound on the terms keeps at most 2^46)
      ok[q] = to_fix128(v[q], E, f[q]);
      if (!WIDE)
        ok[q] = ok[q] && f[q].hi == (unsigned long long)((long long)f[q].lo >> 63) &&
                (f[q].lo + (1ull << 47)) < (1ull << 48);
      if (ok[q]) {
        if (WIDE) add_fix128(h + 2 * (q * nb + bin), f[q]);
        else atomicAdd(h + q * nb + bin, f[q].lo);
      } else {
        atomicAdd(&acc.A[((size_t)cur * Q + q) * nb + bin], v[q]);
      }
    }
    atomicAdd(&hc[bin], 1u);
    if (JK) {
      const int p_s = shp.patch[j];
      if (p_s >= P.n_patch) atomicOr(acc.status, MIA_LC_BAD_PATCH);
      if (p_s >= 0 && p_s < P.n_patch && p_s != cur) {
        const size_t base = (size_t)p_s * Q * nb + bin;
        for (int q = q0; q < q1; ++q) {
          if (ok[q]) add_fix128(acc.B128 + 2 * (base + (size_t)q * nb), f[q]);
          else atomicAdd(&acc.B[base + (size_t)q * nb], v[q]);
        }
        atomicAdd(&acc.cB[(size_t)p_s * nb + bin], 1ull);
      }
    }
  };

  // S+D and SxD terms of a pair from its separation (ux, uy) (any common scale):
  // e+ = -e cos 2(phi_a - phi_s), ex = -e sin 2(phi_a - phi_s) with cos 2phi_s =
  // (ux^2 - uy^2) / q, sin 2phi_s = 2 ux uy / q, q = ux^2 + uy^2; the shape's
  // w_s e cos 2phi_a, w_s e sin 2phi_a come precomputed (k_lc_scatter).  1/q is an
  // FP32 seed and one Newton step (relative error ~1e-14 of the term).
  auto shape_terms = [&](int j, double w_n, double ux, double uy, double& sp, double& sx) {
    sp = sx = 0.0;
    const double ux2 = ux * ux;
    const double qd = fma(uy, uy, ux2);
    if (!(qd > 0.0)) return;                   // r_p = 0: the reference's NaN terms are set to 0
    double r;
    if (qd > 1e-30 && qd < 1e30) {
      r = (double)__frcp_rn((float)qd);
      r = r * fma(-qd, r, 2.0);
    } else {
      r = 1.0 / qd;
    }
    const double A = fma(-uy, uy, ux2), B = (ux + ux) * uy;
    const double k = -w_n * r;
    const double wa = shp.aux1[j], wb = shp.aux2[j];
    sp = k * fma(wa, A, wb * B);
    sx = k * fma(wb, A, -(wa * B));
  };

  // One queued survivor per valid lane: e.z >= 0 is its bin (decided in
  // FP32); e.z < 0 means a decision fell in the guard band: the reference's
  // exact sequence decides (measure_w_lightcone.py:137-172,
  // measure_m_lightcone.py:140-176).
  auto process = [&](bool valid, int4 e) {
    if (!valid) return;
    const int j = e.x, ip = e.y;
    const double ra_n = pos.ra[ip], dec_n = pos.dec[ip], chi_n = pos.chi[ip];
    const double ra_s = shp.ra[j], dec_s = shp.dec[j], chi_s = shp.chi[j];
    const double dra = __dsub_rn(ra_s, ra_n), ddec = __dsub_rn(dec_s, dec_n);
    int bin = e.z;
    double ux, uy;
    if (bin >= 0) {
      ux = dra * pos.aux1[ip];
      uy = ddec * pos.aux2[ip];
    } else {
      const double los = __dsub_rn(chi_s, chi_n);
      const double dra_e = __dmul_rn(__ddiv_rn(dra, 180.0), 3.141592653589793);
      const double ddec_e = __dmul_rn(__ddiv_rn(ddec, 180.0), 3.141592653589793);
      const double dx_e = __dmul_rn(__dmul_rn(dra_e, chi_n), pos.aux0[ip]);
      const double dy_e = __dmul_rn(ddec_e, chi_n);
      const double dxh = P.h_extra != 1.0 ? __dmul_rn(dx_e, P.h_extra) : dx_e;
      const double dyh = P.h_extra != 1.0 ? __dmul_rn(dy_e, P.h_extra) : dy_e;
      const double qp = __dadd_rn(__dmul_rn(dxh, dxh), __dmul_rn(dyh, dyh));
      ux = dxh;
      uy = dyh;
      int ib, jb;
      if (KIND == MIA_KIND_W) {
        ib = lookup(s_qbr, s_qbn, P.n_qbreak, qp);
        if (ib == -1) return;
        jb = lookup(s_pbr, s_pbn, P.n_pbreak, los);
        if (jb == -1) return;
      } else {
        if (!(__dsqrt_rn(qp) > P.rp_cut)) return;
        const double q = __dadd_rn(__dadd_rn(__dmul_rn(dx_e, dx_e), __dmul_rn(dy_e, dy_e)), __dmul_rn(los, los));
        ib = lookup(s_qbr, s_qbn, P.n_qbreak, q);
        if (ib == -1) return;
        jb = lookup(s_pbr, s_pbn, P.n_pbreak, __ddiv_rn(los, __dsqrt_rn(q)));
        if (jb == -1) return;
      }
      if (ib < 0 || jb < 0) {   // np.add.at would raise IndexError here
        atomicOr(acc.status, MIA_LC_INDEX_ERROR);
        return;
      }
      bin = ib * P.n_p + jb;
    }
    const double w_n = pos.w[ip];
    double sp = 0.0, sx = 0.0;
    if (SHAPES) shape_terms(j, w_n, ux, uy, sp, sx);
    accumulate(j, bin, UNIT ? 1.0 : __dmul_rn(w_n, shp.w[j]), sp, sx);
  };

  auto drain = [&]() {   // process what is queued (fewer than 32 entries)
    __syncwarp();
    process(lane < cnt, queue[lane]);
    cnt = 0;
    __syncwarp();
  };

  const float h2f = (float)P.h2, rc2f = (float)(P.rp_cut * P.rp_cut);
  for (;;) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(acc.next, (unsigned)kLcChunk);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((long long)base >= P.n_pos) break;
    const long long stop = min((long long)base + kLcChunk, P.n_pos);
    for (long long ip = base; ip < stop; ++ip) {
      const int p_n = JK ? pos.patch[ip] : 0;
      if (JK && (p_n < 0 || p_n >= P.n_patch)) {   // a position must belong to a patch
        if (lane == 0) atomicOr(acc.status, MIA_LC_BAD_PATCH);
        continue;
      }
      if (p_n != cur) {
        drain();
        flush_hist(cur);
        cur = p_n;
      }
      const double w_n = pos.w[ip];
      const LcWin wn = win[ip];
      const int d0 = wn.d0, d1 = wn.d1, a0 = wn.a0, a1 = wn.a1, c0 = wn.c0, c1 = wn.c1;
      const float kx = wn.kx, ky = wn.ky, gq = wn.gq, gqp = wn.gqp, gmu = wn.gmu, gl = wn.gl;
      const float4 nhl = pos.hl[ip];
      const float2 nch = pos.chl[ip];
      // the window's rows, (DEC band, distance slab) pairs with their RA
      // ranges, are read 32 at a time: lane k sets up row sb + k (its shape
      // range in cell order), a warp scan gives the rows' offsets, and the
      // warp then walks the concatenated candidates 32 at a time, so no lane
      // idles at the end of a row
      const int nc = c1 - c0 + 1, nseg = (d1 - d0 + 1) * nc;
      for (int sb = 0; sb < nseg; sb += 32) {
        int sj0 = 0, slen = 0;
        if (sb + lane < nseg) {
          const int s = sb + lane, d = d0 + s / nc, c = c0 + s % nc;
          // a shape in DEC band d is at least `gap` cells from the position in
          // DEC, so within r_lim it is at most sra sqrt(1 - (gap / sdec)^2)
          // cells away in RA (the window's ellipse); FP32 with margins of
          // 2e-3 cells and 1e-5 relative keeps the range a superset
          int ra0 = a0, ra1 = a1;
          bool keep = true;
          if (wn.sra >= 0.0f) {
            float gap = 0.0f;
            if (d > 0) gap = fmaxf(gap, (float)d - wn.tdec);
            if (d < P.g.n_dec - 1) gap = fmaxf(gap, wn.tdec - (float)(d + 1));
            const float rr = fmaxf(gap - 2e-3f, 0.0f) / wn.sdec;
            float room = 1.0f - rr * rr;
            if (wn.schi > 0.0f) {
              float gc = 0.0f;
              if (c > 0) gc = fmaxf(gc, (float)c - wn.tchi);
              if (c < P.g.n_chi - 1) gc = fmaxf(gc, wn.tchi - (float)(c + 1));
              const float rc = fmaxf(gc - 2e-3f, 0.0f) / wn.schi;
              room -= rc * rc;
            }
            keep = room > -1e-6f;
            const float wc = wn.sra * sqrtf(fmaxf(room, 0.0f)) * (1.0f + 1e-5f) + 2e-3f;
            // clamped as cell_1d clamps: the end cells also hold what lies beyond
            const int nr = P.g.n_ra - 1;
            ra0 = max(a0, min(nr, max(0, (int)floorf(wn.tra - wc))));
            ra1 = min(a1, min(nr, max(0, (int)floorf(wn.tra + wc))));
            keep = keep && ra0 <= ra1;
          }
          if (keep) {
            const int row = (d * P.g.n_chi + c) * P.g.n_ra;
            sj0 = start[row + ra0];
            slen = start[row + ra1 + 1] - sj0;
          }
        }
        int incl = slen;   // inclusive prefix of the row lengths over the lanes
        for (int of = 1; of < 32; of <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, of);
          if (lane >= of) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int seg = 0;       // this lane's row (lane index of its setup), non-decreasing
        for (int vb = 0; vb < total; vb += 32) {
          const int v = vb + lane;
          // move each lane to the row holding candidate v (warp-uniform loop:
          // every lane takes part in the shuffles)
          for (;;) {
            const int end = __shfl_sync(0xffffffffu, incl, seg);
            const bool adv = v < total && v >= end;
            if (!__any_sync(0xffffffffu, adv)) break;
            if (adv) ++seg;
          }
          const int base_j = __shfl_sync(0xffffffffu, sj0, seg);
          const int before = __shfl_sync(0xffffffffu, incl - slen, seg);
          const int j = base_j + (v - before);
          bool take = false;   // binned (bin decided) or in the guard band
          bool near = false;
          int bin = -1;
          if (v < total) {
            const float4 s4 = shp.hl[j];
            const float2 sc = shp.chl[j];
            const float ax = ((s4.x - nhl.x) + (s4.y - nhl.y)) * kx;
            const float ay = ((s4.z - nhl.z) + (s4.w - nhl.w)) * ky;
            const float lf = (sc.x - nch.x) + (sc.y - nch.y);
            const float qn = ax * ax + ay * ay;
            int ib = -1, jb = -1;
            if (KIND == MIA_KIND_W) {
              if (qn <= P.qf_hi && lf >= P.los_lo && lf <= P.los_hi) {
                jb = lookup_f(s_pbf, s_pbn, P.n_pbreak, lf, lf * P.pa + P.pb, kRelGuard * fabsf(lf) + gl, near);
                if (near || jb != -1) {
                  ib = lookup_f(s_qbf, s_qbn, P.n_qbreak, qn, __log2f(qn) * P.qa + P.qb, kRelGuard * qn + gq, near);
                  take = near || ib != -1;
                }
              }
            } else {
              const float q = qn + lf * lf;
              if (q <= P.qf_hi) {
                bool cut_ok = true;
                if (P.rp_cut >= 0.0) {
                  const float qp = qn * h2f;
                  if (fabsf(qp - rc2f) <= kRelGuard * fmaxf(qp, rc2f) + gqp) near = true;
                  cut_ok = qp > rc2f;
                }
                if (near || cut_ok) {
                  ib = lookup_f(s_qbf, s_qbn, P.n_qbreak, q, __log2f(q) * P.qa + P.qb, kRelGuard * q + gq, near);
                  if (near || ib != -1) {
                    const float rq = rsqrtf(q);
                    const float mu = lf * rq;
                    jb = lookup_f(s_pbf, s_pbn, P.n_pbreak, mu, mu * P.pa + P.pb, kRelGuard + gmu * rq, near);
                    take = true;
                  }
                }
              }
            }
            if (take && !near) {
              if (ib < 0 || jb < 0) {   // np.add.at would raise IndexError here
                atomicOr(acc.status, MIA_LC_INDEX_ERROR);
                take = false;
              } else {
                bin = ib * P.n_p + jb;
              }
            }
            if (!SHAPES && take && !near) {   // counts only: w_p w_s is all there is to add
              accumulate(j, bin, UNIT ? 1.0 : __dmul_rn(w_n, shp.w[j]), 0.0, 0.0);
              take = false;
            }
          }
          const unsigned bal = __ballot_sync(0xffffffffu, take);
          if (bal) {
            if (take) queue[cnt + __popc(bal & ((1u << lane) - 1u))] = make_int4(j, (int)ip, near ? -1 : bin, 0);
            cnt += __popc(bal);
            if (cnt >= 32) {
              __syncwarp();
              const int4 mine = queue[lane];
              __syncwarp();
              const int rest = cnt - 32;
              if (lane < rest) queue[lane] = queue[32 + lane];
              cnt = rest;
              __syncwarp();
              process(true, mine);
            }
          }
          // a step adds at most 64 terms to the partials (32 decided here,
          // 32 from the queue); 1000 steps stay below 2^16 terms of < 2^47
          steps += 2;
          if (steps >= P.flush_steps) {
            flush_hist(cur);
            steps = 0;
          }
        }
      }
    }
  }
  drain();
  flush_hist(cur);
}

// totals and realisations: out[q][0][b] = sum_i A[i][q][b]; out[q][1+i][b] =
// total - A[i] - B[i], in exact 128-bit integers, rounded once (plus the same
// combination of the terms that were not finite); the integer counts likewise.
__device__ __forceinline__ void add128(unsigned long long& lo, unsigned long long& hi, const unsigned long long* v) {
  const unsigned long long l = lo + v[0];
  hi = hi + v[1] + (l < lo ? 1ull : 0ull);
  lo = l;
}
__device__ __forceinline__ void sub128(unsigned long long& lo, unsigned long long& hi, const unsigned long long* v) {
  const unsigned long long l = lo - v[0];
  hi = hi - v[1] - (lo < v[0] ? 1ull : 0ull);
  lo = l;
}

__global__ void k_lc_finish(const unsigned long long* __restrict__ A128, const unsigned long long* __restrict__ B128,
                            const double* __restrict__ A, const double* __restrict__ B,
                            const unsigned long long* __restrict__ cA, const unsigned long long* __restrict__ cB,
                            const unsigned long long* __restrict__ wmax, int wide, int n_patch, int Q, int nb,
                            int unit, double* out, long long* counts) {
  const int P = n_patch > 0 ? n_patch : 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_real = 1 + n_patch;
  if (unit && t < nb) {   // unit weights: DD is the pair count (exact in FP64 below 2^53)
    const int b = t;
    unsigned long long tot = 0;
    for (int i = 0; i < P; ++i) tot += cA[(size_t)i * nb + b];
    out[b] = (double)tot;
    for (int i = 0; i < n_patch; ++i)
      out[(size_t)(1 + i) * nb + b] = (double)(tot - cA[(size_t)i * nb + b] - cB[(size_t)i * nb + b]);
  } else if (t < Q * nb) {
    const int q = t / nb, b = t - q * nb;
    const double inv = ldexp(1.0, -lc_exponent(wmax, wide));
    unsigned long long tl = 0, th = 0;
    double pt = 0.0;
    for (int i = 0; i < P; ++i) {
      const size_t k = ((size_t)i * Q + q) * nb + b;
      add128(tl, th, A128 + 2 * k);
      pt += A[k];
    }
    double* o = out + (size_t)q * n_real * nb;
    o[b] = fix128_value(tl, th, inv) + pt;
    for (int i = 0; i < n_patch; ++i) {
      const size_t k = ((size_t)i * Q + q) * nb + b;
      unsigned long long rl = tl, rh = th;
      sub128(rl, rh, A128 + 2 * k);
      sub128(rl, rh, B128 + 2 * k);
      o[(size_t)(1 + i) * nb + b] = fix128_value(rl, rh, inv) + ((pt - A[k]) - B[k]);
    }
  } else if (t < Q * nb + nb) {
    const int b = t - Q * nb;
    unsigned long long tot = 0;
    for (int i = 0; i < P; ++i) tot += cA[(size_t)i * nb + b];
    counts[b] = (long long)tot;
    for (int i = 0; i < n_patch; ++i)
      counts[(size_t)(1 + i) * nb + b] = (long long)(tot - cA[(size_t)i * nb + b] - cB[(size_t)i * nb + b]);
  }
}

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// a sample in cell order: 7 double arrays, the patch labels, the FP32 hi/lo
// copies; 11 (n + 8) doubles in all, every array 16-byte aligned
constexpr size_t kSortedDoubles = 11;

LcSorted carve(unsigned char* base, long long n) {
  LcSorted s;
  const size_t nn = (size_t)n + 8;
  double* d = reinterpret_cast<double*>(base);
  s.ra = d;
  s.dec = d + nn;
  s.chi = d + 2 * nn;
  s.w = d + 3 * nn;
  s.aux0 = d + 4 * nn;
  s.aux1 = d + 5 * nn;
  s.aux2 = d + 6 * nn;
  s.patch = reinterpret_cast<int*>(d + 7 * nn);
  s.hl = reinterpret_cast<float4*>(d + 8 * nn);
  s.chl = reinterpret_cast<float2*>(d + 10 * nn);
  return s;
}

// per warp: the survivor queue, hq * nb 64-bit partial sums, nb u32 counts
size_t lc_per_warp(int hq, int nb, int wide) {
  return (size_t)kQueue * 16 + (size_t)hq * nb * (wide ? 16 : 8) + (size_t)(nb + 1) / 2 * 8;
}
constexpr size_t kLcFixedSmem = kLcTableBytes + 16;
constexpr size_t kLcSmemBudget = 200 * 1024;

template <int KIND, int SHAPES, int JK, int UNIT, int WIDE>
cudaError_t launch_lc_pairs(const LcParams& P, const LcTables& T, const LcSorted& pos, const LcSorted& shp,
                            const int* start, const LcWin* win, const LcAcc& acc, int warps, size_t smem, int num_sms,
                            cudaStream_t st) {
  auto kern = k_lc_pairs<KIND, SHAPES, JK, UNIT, WIDE>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const long long want = (P.n_pos + kLcChunk - 1) / kLcChunk;
  long long blocks = std::min<long long>((long long)num_sms * per_sm, (want + warps - 1) / warps);
  if (blocks < 1) blocks = 1;
  kern<<<(int)blocks, warps * 32, smem, st>>>(P, T, pos, shp, start, win, acc);
  return cudaGetLastError();
}

}  // namespace

bool lc_plan(const mia_lc_config* c, long long n_pos, long long n_shape, LcPlan* p, const char** why) {
  memset(p, 0, sizeof(*p));
  if (!c) { *why = "null config"; return false; }
  if (c->kind != MIA_KIND_W && c->kind != MIA_KIND_MULTIPOLES) { *why = "kind"; return false; }
  if (c->n_r < 1 || c->n_p < 1 || c->n_r > MIA_MAX_BINS_R || c->n_p > MIA_MAX_BINS_P) { *why = "bin counts"; return false; }
  if (c->n_patch < 0 || c->n_patch > 100000) { *why = "n_patch"; return false; }
  if (c->n_qbreak < 0 || c->n_qbreak > MIA_MAX_BREAKS || c->n_pbreak < 0 || c->n_pbreak > MIA_MAX_BREAKS ||
      !c->q_break || !c->q_bin || !c->p_break || !c->p_bin) { *why = "bin tables"; return false; }
  if (c->n_ra < 1 || c->n_dec < 1 || c->n_chi < 1 || !(c->ra_cell > 0) || !(c->dec_cell > 0) || !(c->chi_cell > 0) ||
      !std::isfinite(c->ra0) || !std::isfinite(c->dec0) || !std::isfinite(c->chi0)) {
    *why = "cell grid"; return false;
  }
  if (!(c->r_lim > 0) || !std::isfinite(c->r_lim) || !(c->h_extra > 0) || !std::isfinite(c->h_extra)) {
    *why = "r_lim / h_extra"; return false;
  }
  if (n_pos < 0 || n_shape < 0 || n_pos > (1ll << 31) - 64 || n_shape > (1ll << 31) - 64) { *why = "sample sizes"; return false; }
  p->n_cells = (long long)c->n_ra * c->n_dec * c->n_chi;
  if (p->n_cells > (1ll << 27)) { *why = "too many cells"; return false; }
  p->Q = c->with_shapes ? 3 : 1;
  p->hq = (!c->with_shapes && c->unit_weights) ? 0 : p->Q;
  p->wide = (c->wide_sums && !c->unit_weights) ? 1 : 0;
  p->nb = c->n_r * c->n_p;
  p->P = c->n_patch > 0 ? c->n_patch : 1;
  const size_t per_warp = lc_per_warp(p->hq, p->nb, p->wide);
  if (kLcFixedSmem + per_warp > kLcSmemBudget) { *why = "too many bins for the lightcone counter"; return false; }
  p->warps = (int)std::min<size_t>(kLcMaxWarps, (kLcSmemBudget - kLcFixedSmem) / per_warp);
  p->smem = kLcFixedSmem + (size_t)p->warps * per_warp;
  p->n_tiles = (int)((p->n_cells + kScanTile - 1) / kScanTile) + 1;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += al(bytes); return at; };
  p->off_scount = take((size_t)(p->n_cells + 1) * 4);
  p->off_sstart = take((size_t)(p->n_cells + 2) * 4);
  p->off_sfill = take((size_t)(p->n_cells + 1) * 4);
  p->off_pcount = take((size_t)(p->n_cells + 1) * 4);
  p->off_pstart = take((size_t)(p->n_cells + 2) * 4);
  p->off_pfill = take((size_t)(p->n_cells + 1) * 4);
  p->off_tiles = take((size_t)p->n_tiles * 4);
  p->off_scell = take((size_t)n_shape * 4 + 4);
  p->off_pcell = take((size_t)n_pos * 4 + 4);
  p->off_shp = take(((size_t)n_shape + 8) * kSortedDoubles * 8);
  p->off_pos = take(((size_t)n_pos + 8) * kSortedDoubles * 8);
  p->off_A = take((size_t)p->P * p->Q * p->nb * 8);
  p->off_B = take((size_t)c->n_patch * p->Q * p->nb * 8 + 8);
  p->off_cA = take((size_t)p->P * p->nb * 8);
  p->off_cB = take((size_t)c->n_patch * p->nb * 8 + 8);
  p->off_A128 = take((size_t)p->P * p->Q * p->nb * 16);
  p->off_B128 = take((size_t)c->n_patch * p->Q * p->nb * 16 + 16);
  p->off_wmax = take(16);
  p->off_win = take(((size_t)n_pos + 1) * sizeof(LcWin));
  p->off_next = take(256);
  p->total = o;
  return true;
}

cudaError_t launch_lc(const mia_lc_config* cfg, const LcPlan& p, const mia_lc_sample& pos,
                      const mia_lc_sample& shp, void* workspace, double* out, int64_t* counts, uint32_t* status,
                      int num_sms, cudaStream_t st) {
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  int* scount = reinterpret_cast<int*>(ws + p.off_scount);
  int* sstart = reinterpret_cast<int*>(ws + p.off_sstart);
  int* sfill = reinterpret_cast<int*>(ws + p.off_sfill);
  int* pcount = reinterpret_cast<int*>(ws + p.off_pcount);
  int* pstart = reinterpret_cast<int*>(ws + p.off_pstart);
  int* pfill = reinterpret_cast<int*>(ws + p.off_pfill);
  int* tiles = reinterpret_cast<int*>(ws + p.off_tiles);
  int* scell = reinterpret_cast<int*>(ws + p.off_scell);
  int* pcell = reinterpret_cast<int*>(ws + p.off_pcell);
  const LcSorted S = carve(ws + p.off_shp, shp.n);
  const LcSorted Ps = carve(ws + p.off_pos, pos.n);
  LcAcc acc;
  acc.A128 = reinterpret_cast<unsigned long long*>(ws + p.off_A128);
  acc.B128 = reinterpret_cast<unsigned long long*>(ws + p.off_B128);
  unsigned long long* wmax = reinterpret_cast<unsigned long long*>(ws + p.off_wmax);
  acc.wmax = wmax;
  acc.A = reinterpret_cast<double*>(ws + p.off_A);
  acc.B = reinterpret_cast<double*>(ws + p.off_B);
  acc.cA = reinterpret_cast<unsigned long long*>(ws + p.off_cA);
  acc.cB = reinterpret_cast<unsigned long long*>(ws + p.off_cB);
  acc.next = reinterpret_cast<unsigned*>(ws + p.off_next);
  acc.status = status;

  LcGrid g;
  g.ra0 = cfg->ra0; g.inv_ra = 1.0 / cfg->ra_cell; g.n_ra = cfg->n_ra;
  g.dec0 = cfg->dec0; g.inv_dec = 1.0 / cfg->dec_cell; g.n_dec = cfg->n_dec;
  g.chi0 = cfg->chi0; g.inv_chi = 1.0 / cfg->chi_cell; g.n_chi = cfg->n_chi;

  cudaError_t e;
  const size_t cells_b = (size_t)(p.n_cells + 1) * 4;
  if ((e = cudaMemsetAsync(scount, 0, cells_b, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(pcount, 0, cells_b, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(ws + p.off_A, 0, p.total - p.off_A, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(status, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
  auto grid_for = [&](long long n) {
    const long long b = (n + 255) / 256;
    return (int)std::max(1ll, std::min(b, (long long)num_sms * 8));
  };
  if (shp.n > 0) k_lc_cells<<<grid_for(shp.n), 256, 0, st>>>(shp.ra, shp.dec, shp.chi, shp.n, g, scell, scount);
  if (pos.n > 0) k_lc_cells<<<grid_for(pos.n), 256, 0, st>>>(pos.ra, pos.dec, pos.chi, pos.n, g, pcell, pcount);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = exclusive_scan(scount, p.n_cells, sstart, tiles, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(sfill, sstart, (size_t)p.n_cells * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if ((e = exclusive_scan(pcount, p.n_cells, pstart, tiles, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(pfill, pstart, (size_t)p.n_cells * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if (shp.n > 0) k_lc_scatter<<<grid_for(shp.n), 256, 0, st>>>(shp, shp.n, scell, sfill, S, 0, cfg->with_shapes, wmax + 1);
  if (pos.n > 0) k_lc_scatter<<<grid_for(pos.n), 256, 0, st>>>(pos, pos.n, pcell, pfill, Ps, 1, 0, wmax);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;

  LcParams P;
  P.n_r = cfg->n_r; P.n_p = cfg->n_p; P.nb = p.nb; P.n_patch = cfg->n_patch; P.Q = p.Q;
  P.n_qbreak = cfg->n_qbreak; P.n_pbreak = cfg->n_pbreak;
  P.h_extra = cfg->h_extra; P.h2 = cfg->h_extra * cfg->h_extra; P.rp_cut = cfg->rp_cut; P.r_lim = cfg->r_lim;
  P.pi_lo = cfg->pi_lo; P.pi_hi = cfg->pi_hi;
  P.qf_hi = (float)(cfg->r_lim * cfg->r_lim * (1.0 + 1e-4));
  {
    const double mpi = 1e-4 * (fabs(cfg->pi_lo) + fabs(cfg->pi_hi)) + 1e-6;
    P.los_lo = (float)(cfg->pi_lo - mpi);
    P.los_hi = (float)(cfg->pi_hi + mpi);
  }
  P.g = g;
  P.n_pos = pos.n;
  P.unit = cfg->unit_weights ? 1 : 0;
  P.hq = p.hq;
  // MIA_LC_FLUSH_STEPS=<n> flushes the warp partials more often (tests of the
  // flush path; the default is the largest interval the 64-bit partials allow)
  P.flush_steps = kLcFlushSteps;
  if (const char* env = std::getenv("MIA_LC_FLUSH_STEPS")) {
    const int v = std::atoi(env);
    if (v >= 2 && v < kLcFlushSteps) P.flush_steps = v;
  }
  // first guesses of the table intervals: breaks 0 and n-1 map to 1 and n
  auto affine = [](const double* br, int n, bool logq, float* a, float* b) {
    *a = 0.0f;
    *b = 0.0f;
    if (n < 2) return;
    const double x0 = logq ? log2(br[0] > 0 ? br[0] : 1e-300) : br[0];
    const double x1 = logq ? log2(br[n - 1] > 0 ? br[n - 1] : 1e-300) : br[n - 1];
    if (!(x1 > x0) || !std::isfinite(x0) || !std::isfinite(x1)) return;
    const double sl = (n - 1) / (x1 - x0);
    *a = (float)sl;
    *b = (float)(1.0 - sl * x0);
  };
  affine(cfg->q_break, cfg->n_qbreak, true, &P.qa, &P.qb);
  affine(cfg->p_break, cfg->n_pbreak, false, &P.pa, &P.pb);
  LcWin* win = reinterpret_cast<LcWin*>(ws + p.off_win);
  if (pos.n > 0) {
    if (cfg->kind == MIA_KIND_W)
      k_lc_windows<MIA_KIND_W><<<grid_for(pos.n), 256, 0, st>>>(P, Ps, win);
    else
      k_lc_windows<MIA_KIND_MULTIPOLES><<<grid_for(pos.n), 256, 0, st>>>(P, Ps, win);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  LcTables T;
  for (int i = 0; i < MIA_MAX_BREAKS; ++i) {
    T.qbr[i] = i < cfg->n_qbreak ? cfg->q_break[i] : 0.0;
    T.pbr[i] = i < cfg->n_pbreak ? cfg->p_break[i] : 0.0;
  }
  for (int i = 0; i <= MIA_MAX_BREAKS; ++i) {
    T.qbn[i] = i <= cfg->n_qbreak ? cfg->q_bin[i] : -1;
    T.pbn[i] = i <= cfg->n_pbreak ? cfg->p_bin[i] : -1;
  }
  if (pos.n > 0 && shp.n > 0) {
    const bool jk = cfg->n_patch > 0;
    const int w = p.warps;
#define MIA_LC_CASE(K, S_, J, U, W)                                                                 \
  if (cfg->kind == K && (cfg->with_shapes != 0) == (S_ != 0) && jk == (J != 0) && unit == (U != 0) && \
      (p.wide != 0) == (W != 0))                                                                     \
    e = launch_lc_pairs<K, S_, J, U, W>(P, T, Ps, S, sstart, win, acc, w, p.smem, num_sms, st);
#define MIA_LC_CASES(K, S_, J) MIA_LC_CASE(K, S_, J, 0, 0) MIA_LC_CASE(K, S_, J, 0, 1) MIA_LC_CASE(K, S_, J, 1, 0)
    const bool unit = cfg->unit_weights != 0;
    e = cudaErrorInvalidValue;
    MIA_LC_CASES(MIA_KIND_W, 0, 0) MIA_LC_CASES(MIA_KIND_W, 0, 1) MIA_LC_CASES(MIA_KIND_W, 1, 0)
    MIA_LC_CASES(MIA_KIND_W, 1, 1) MIA_LC_CASES(MIA_KIND_MULTIPOLES, 0, 0) MIA_LC_CASES(MIA_KIND_MULTIPOLES, 0, 1)
    MIA_LC_CASES(MIA_KIND_MULTIPOLES, 1, 0) MIA_LC_CASES(MIA_KIND_MULTIPOLES, 1, 1)
#undef MIA_LC_CASES
#undef MIA_LC_CASE
    if (e != cudaSuccess) return e;
  }
  const int n_thr = (p.Q + 1) * p.nb;
  k_lc_finish<<<(n_thr + 255) / 256, 256, 0, st>>>(acc.A128, acc.B128, acc.A, acc.B, acc.cA, acc.cB, wmax, p.wide,
                                                    cfg->n_patch, p.Q, p.nb, cfg->unit_weights ? 1 : 0, out,
                                                    reinterpret_cast<long long*>(counts));
  return cudaGetLastError();
}

}  // namespace mia
