// Pair-counting kernels: the persistent cell-pair kernel in its plain FP64 and
// mixed FP32 forms, and the FP64 re-test of near-edge pairs.
//
// Reference hot loop replaced: the per-shape pair binning and np.add.at
// scatters of _measure_xi_rp_pi_box_jk_batch (measure_w_box_jk.py:581-644) and
// _measure_xi_r_mur_box_jk_batch (measure_m_box_jk.py:608-680), together with
// the KD-tree candidate search that feeds them (:577-580) and the Pool.map over
// shape chunks (:765-780).
//
// Work decomposition: one work unit = up to `shapes_per_unit` shapes of one
// cell that share a jackknife label a.  A block takes a unit from a global
// counter, stages the shapes in shared memory, and streams every position of
// the neighbouring cells (rows of cells along d0 are contiguous in the sorted
// position arrays); each thread owns one position at a time and loops over the
// unit's shapes.  Pair contributions go to block-private shared histograms,
// one per jackknife region b of the positions ("slot"), flushed at the end of
// the unit into the global histograms of all pairs, of region a and of region
// b != a (the attribution rule of measure_w_box_jk.py:625-644).
#include <cstdio>

#include "mia_internal.cuh"

namespace mia {

namespace {

#ifndef MIA_BIN_CACHE
#define MIA_BIN_CACHE 0  // per-thread two-entry cache of bin partials in front of the shared atomics
#endif

constexpr int kRowsPerPass = 512;
constexpr int kSegsPerPass = 2 * kRowsPerPass;

struct SmemLayout {
  size_t tables, slot_of, slot_region, shapes, seg_begin, seg_pref, seg_shift, hist, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Words of histogram state per (slot, bin).
__host__ __device__ inline int hist_words(int mixed, int var) {
  // mixed: cnt, dd lo/hi, sp lo/hi, sx lo/hi (+ var lo/hi)  -- u32 words
  // fp64 : cnt (u32) + dd, sp, sx (+ var) doubles -> counted in u32 words
  return mixed ? (7 + (var ? 2 : 0)) : (1 + 6 + (var ? 2 : 0));
}

struct TablesSmem {
  long long q_key[MIA_MAX_BREAKS];
  int q_bin[MIA_MAX_BREAKS + 1];
  float q_lo32[MIA_MAX_BREAKS];
  float q_hi32[MIA_MAX_BREAKS];
  long long p_key[MIA_MAX_BREAKS];
  int p_bin[MIA_MAX_BREAKS + 1];
  unsigned short lut32[kLut];
};

__host__ __device__ inline SmemLayout smem_layout(int J, int spu, int K, int nb, int mixed, int var) {
  SmemLayout L;
  size_t o = 0;
  L.tables = o;
  o = align16(o + sizeof(TablesSmem));
  L.slot_of = o;
  o = align16(o + sizeof(int) * (size_t)(J + 1));
  L.slot_region = o;
  o = align16(o + sizeof(int) * kMaxSlots);
  L.shapes = o;
  o = align16(o + (size_t)spu * (mixed ? 44 : 56));
  L.seg_begin = o;
  o = align16(o + sizeof(int) * kSegsPerPass);
  L.seg_pref = o;
  o = align16(o + sizeof(int) * (kSegsPerPass + 1));
  L.seg_shift = o;
  o = align16(o + sizeof(int) * kSegsPerPass);
  L.hist = o;
  o = align16(o + sizeof(unsigned) * (size_t)K * nb * hist_words(mixed, var) + 16);
  L.total = o;
  return L;
}

// ---- accumulation helpers ---------------------------------------------------

// 64-bit fixed-point add built from native 32-bit shared atomics: the low word
// takes the value, a carry or borrow out of it goes to the high word.
__device__ __forceinline__ void acc_fixed(unsigned* lo, int* hi, int idx, int v) {
  unsigned old = atomicAdd(&lo[idx], (unsigned)v);
  unsigned nw = old + (unsigned)v;
  int d = (v < 0 ? -1 : 0) + (nw < old ? 1 : 0);
  if (d) atomicAdd(&hi[idx], d);
}

// Add a signed 64-bit fixed-point partial to a (low word, high word) pair.
__device__ __forceinline__ void add64_shared(unsigned* lo, int* hi, int idx, long long v) {
  const unsigned vlo = (unsigned)(unsigned long long)v;
  int vhi = (int)(v >> 32);
  const unsigned old = atomicAdd(&lo[idx], vlo);
  vhi += (old + vlo < old) ? 1 : 0;
  if (vhi) atomicAdd(&hi[idx], vhi);
}

__device__ __forceinline__ double fixed_value(const unsigned* lo, const int* hi, int idx, double inv) {
  long long v = ((long long)hi[idx] << 32) + (long long)lo[idx];
  return (double)v * inv;
}

// Direct global accumulation (pairs whose position region has no slot, and the
// FP64 edge re-test).
__device__ __forceinline__ void acc_global(const Out& o, int nb, int J, int a, int b, int bin, double dd, double sp,
                                           double sx, double var, int want_var) {
  atomicAdd(&o.npairs[bin], 1ULL);
  atomicAdd(&o.dd[bin], dd);
  atomicAdd(&o.splus[bin], sp);
  atomicAdd(&o.scross[bin], sx);
  if (want_var) atomicAdd(&o.variance[bin], var);
  if (J > 0) {
    size_t ia = (size_t)(1 + a) * nb + bin;
    atomicAdd(&o.npairs[ia], 1ULL);
    atomicAdd(&o.dd[ia], dd);
    atomicAdd(&o.splus[ia], sp);
    if (b != a) {
      size_t ib = (size_t)(1 + b) * nb + bin;
      atomicAdd(&o.npairs[ib], 1ULL);
      atomicAdd(&o.dd[ib], dd);
      atomicAdd(&o.splus[ib], sp);
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

// ---- the persistent pair kernel ----------------------------------------------

template <int MIXED, int VAR, int KIND, int FULL>
__global__ void __launch_bounds__(kThreads) k_pairs(Params P, Work w, Out o, int K) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x;
  const int nb = P.nb;
  const SmemLayout SL = smem_layout(P.J, P.shapes_per_unit, K, nb, MIXED, VAR);
  TablesSmem& T = *reinterpret_cast<TablesSmem*>(smem + SL.tables);
  int* slot_of = reinterpret_cast<int*>(smem + SL.slot_of);
  int* slot_region = reinterpret_cast<int*>(smem + SL.slot_region);
  int* seg_begin = reinterpret_cast<int*>(smem + SL.seg_begin);
  int* seg_pref = reinterpret_cast<int*>(smem + SL.seg_pref);
  int* seg_shift = reinterpret_cast<int*>(smem + SL.seg_shift);
  unsigned* hist = reinterpret_cast<unsigned*>(smem + SL.hist);
  const int KB = K * nb;

  __shared__ int s_wu;
  __shared__ int s_nslots;
  __shared__ int s_scan[32];
  __shared__ int s_total;

  // tables -> shared
  {
    const Tables& G = *w.tables;
    for (int i = tid; i < MIA_MAX_BREAKS; i += blockDim.x) {
      T.q_key[i] = G.q_key[i];
      T.q_lo32[i] = G.q_lo32[i];
      T.q_hi32[i] = G.q_hi32[i];
      T.p_key[i] = G.p_key[i];
    }
    for (int i = tid; i < MIA_MAX_BREAKS + 1; i += blockDim.x) {
      T.q_bin[i] = G.q_bin[i];
      T.p_bin[i] = G.p_bin[i];
    }
    if (MIXED)
      for (int i = tid; i < kLut; i += blockDim.x) T.lut32[i] = G.lut32[i];
    for (int i = tid; i <= P.J; i += blockDim.x) slot_of[i] = -1;
    if (tid == 0) s_nslots = 0;
  }
  const double twoR = 2.0 * (w.reg.s1[P.J] / w.reg.s2[P.J]);
  const unsigned long long n_wu = w.status->n_wu;
  // fixed-point scale 2^S with |term| * 2^S <= 2^30 for every pair term
  float fixed_scale = 1.0f;
  double fixed_inv = 1.0;
  if (MIXED) {
    double m = __longlong_as_double((long long)w.status->maxw_bits) *
               __longlong_as_double((long long)w.status->maxws_bits);
    if (!(m > 0.0) || !(m < 1e300)) m = 1.0;
    int S = (int)floor(log2(1073741824.0 / m));
    S = S > 40 ? 40 : (S < -60 ? -60 : S);
    fixed_scale = ldexpf(1.0f, S);
    fixed_inv = ldexp(1.0, -S);
  }
  __syncthreads();

  // views of the per-bin state
  unsigned* h_cnt = hist;
  unsigned *dd_lo = nullptr, *sp_lo = nullptr, *sx_lo = nullptr, *vr_lo = nullptr;
  int *dd_hi = nullptr, *sp_hi = nullptr, *sx_hi = nullptr, *vr_hi = nullptr;
  double *dd_d = nullptr, *sp_d = nullptr, *sx_d = nullptr, *vr_d = nullptr;
  if (MIXED) {
    dd_lo = hist + KB;
    dd_hi = reinterpret_cast<int*>(hist + 2 * KB);
    sp_lo = hist + 3 * KB;
    sp_hi = reinterpret_cast<int*>(hist + 4 * KB);
    sx_lo = hist + 5 * KB;
    sx_hi = reinterpret_cast<int*>(hist + 6 * KB);
    if (VAR) {
      vr_lo = hist + 7 * KB;
      vr_hi = reinterpret_cast<int*>(hist + 8 * KB);
    }
  } else {
    // doubles start at an 8-byte boundary after the counts
    size_t off = align16(sizeof(unsigned) * (size_t)KB);
    double* base = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(hist) + off);
    dd_d = base;
    sp_d = base + KB;
    sx_d = base + 2 * KB;
    if (VAR) vr_d = base + 3 * KB;
  }
  const int hist_u32 = MIXED ? KB * hist_words(1, VAR) : (int)(align16(sizeof(unsigned) * (size_t)KB) / 4) + KB * 2 * (3 + VAR);

  // row enumeration extents (line-of-sight dimension d2 and projected d1)
  int lo1 = P.full[1] ? -(P.n[1] / 2) : -P.R[1];
  int N1 = P.full[1] ? P.n[1] : 2 * P.R[1] + 1;
  int lo2 = P.full[2] ? -(P.n[2] / 2) : -P.R[2];
  int N2 = P.full[2] ? P.n[2] : 2 * P.R[2] + 1;
  const int n_rows = N1 * N2;
  const double r2proj = P.range_proj * P.range_proj;
  const double r2los = P.range_los * P.range_los;

  unsigned long long my_binned = 0;

  while (true) {
    if (tid == 0) s_wu = (int)atomicAdd(&w.status->wu_next, 1ULL);
    __syncthreads();
    const int wi = s_wu;
    if ((unsigned long long)wi >= n_wu) break;
    const WorkUnit u = w.wu[wi];
    int c[3];
    {
      long long t = u.cell;
      c[0] = (int)(t % P.n[0]);
      t /= P.n[0];
      c[1] = (int)(t % P.n[1]);
      c[2] = (int)(t / P.n[1]);
    }
    // -- slot map for the jackknife regions around this cell
    if (tid == 0) {
      for (int k = 0; k < s_nslots; ++k) slot_of[slot_region[k]] = -1;
      int ns = 0;
      if (P.J == 0) {
        slot_of[0] = 0;
        slot_region[0] = 0;
        ns = 1;
      } else {
        int sets[3][16];
        int cnt[3] = {0, 0, 0};
        for (int k = 0; k < 3; ++k) {
          int lo = P.full[k] ? -(P.n[k] / 2) : -P.R[k];
          int N = P.full[k] ? P.n[k] : 2 * P.R[k] + 1;
          for (int d = 0; d < N && cnt[k] < 16; ++d) {
            int cc = wrapi(((c[k] + lo + d) % P.n[k] + P.n[k]) % P.n[k], P.n[k]);
            int sb = (int)((long long)cc * P.n_sub / P.n[k]);
            bool seen = false;
            for (int j = 0; j < cnt[k]; ++j) seen |= sets[k][j] == sb;
            if (!seen) sets[k][cnt[k]++] = sb;
          }
        }
        for (int i0 = 0; i0 < cnt[0]; ++i0)
          for (int i1 = 0; i1 < cnt[1]; ++i1)
            for (int i2 = 0; i2 < cnt[2]; ++i2) {
              int sub[3];
              sub[P.axis[0]] = sets[0][i0];
              sub[P.axis[1]] = sets[1][i1];
              sub[P.axis[2]] = sets[2][i2];
              int reg = (sub[0] * P.n_sub + sub[1]) * P.n_sub + sub[2];
              if (slot_of[reg] < 0 && ns < K) {
                slot_of[reg] = ns;
                slot_region[ns++] = reg;
              }
            }
        if (slot_of[0] < 0 && ns < K) {
          slot_of[0] = ns;
          slot_region[ns++] = 0;
        }
      }
      s_nslots = ns;
    }
    for (int i = tid; i < hist_u32; i += blockDim.x) hist[i] = 0u;
    // -- shapes of the unit -> shared
    const int S = u.count;
    if (MIXED) {
      // stage the shapes ordered by line-of-sight coordinate: consecutive
      // shapes then tend to share a (r_p, Pi) bin with a given position,
      // which the per-thread accumulator cache below exploits
      float4* A = reinterpret_cast<float4*>(smem + SL.shapes);
      float4* B = A + P.shapes_per_unit;
      float2* C = reinterpret_cast<float2*>(B + P.shapes_per_unit);
      int* I = reinterpret_cast<int*>(C + P.shapes_per_unit);
      float* zs = reinterpret_cast<float*>(seg_begin);  // free until the segments are built
      float4 ra = make_float4(0.f, 0.f, 0.f, 0.f), rb = ra;
      float2 rc = make_float2(0.f, 0.f);
      float z = 0.f;
      const int g = u.begin + tid;
      if (tid < S) {
        ra = make_float4(w.sxh[g], w.syh[g], w.szh[g], w.swsf[g]);
        rb = make_float4(w.sxl[g], w.syl[g], w.szl[g], w.swef[g]);
        rc = make_float2(w.saxf[g], w.sayf[g]);
        z = ra.z + rb.z;
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
      }
    } else {
      double* D = reinterpret_cast<double*>(smem + SL.shapes);
      const int M = P.shapes_per_unit;
      for (int i = tid; i < S; i += blockDim.x) {
        int g = u.begin + i;
        D[i] = w.sx[g];
        D[M + i] = w.sy[g];
        D[2 * M + i] = w.sz[g];
        D[3 * M + i] = w.sax[g];
        D[4 * M + i] = w.say[g];
        D[5 * M + i] = w.se[g];
        D[6 * M + i] = w.sws[g];
      }
    }
    __syncthreads();

    for (int pass = 0; pass < n_rows; pass += kRowsPerPass) {
      // -- segments of this pass: two per row (a row may wrap around d0)
      for (int rr = tid; rr < kRowsPerPass; rr += blockDim.x) {
        int r = pass + rr;
        int len0 = 0, len1 = 0, b0 = 0, b1 = 0, sh0 = 0, sh1 = 0;
        if (r < n_rows) {
          int d1 = lo1 + r % N1, d2 = lo2 + r / N1;
          int g1 = abs(d1) - 1, g2 = abs(d2) - 1;
          double gap1 = g1 > 0 ? g1 * P.s[1] : 0.0;
          double gap2 = g2 > 0 ? g2 * P.s[2] : 0.0;
          double rem;
          bool ok;
          if (KIND == MIA_KIND_W) {
            ok = gap1 * gap1 <= r2proj && gap2 * gap2 <= r2los;
            rem = r2proj - gap1 * gap1;
          } else {
            rem = r2proj - gap1 * gap1 - gap2 * gap2;
            ok = rem >= 0.0;
          }
          if (ok) {
            int u1 = c[1] + d1, u2 = c[2] + d2;
            int sh1d = u1 < 0 ? -1 : (u1 >= P.n[1] ? 1 : 0);
            int sh2d = u2 < 0 ? -1 : (u2 >= P.n[2] ? 1 : 0);
            int cc1 = wrapi(u1, P.n[1]), cc2 = wrapi(u2, P.n[2]);
            int xlo, xhi;
            if (P.full[0]) {
              xlo = -(P.n[0] / 2);
              xhi = P.n[0] - P.n[0] / 2 - 1;
            } else {
              double r0 = sqrt(rem > 0.0 ? rem : 0.0);
              int R0 = (int)ceil(r0 / P.s[0] * (1.0 + 1e-9));
              if (R0 > P.R[0]) R0 = P.R[0];
              xlo = -R0;
              xhi = R0;
            }
            long long rowbase = ((long long)cc2 * P.n[1] + cc1) * P.n[0];
            int a0 = c[0] + xlo, a1 = c[0] + xhi;
            int code_yz = 3 * (sh1d + 1) + 9 * (sh2d + 1);
            if (a0 < 0) {
              int lo_c = a0 + P.n[0];
              b0 = w.pstart[rowbase + lo_c];
              len0 = w.pstart[rowbase + P.n[0]] - b0;
              sh0 = code_yz + 0;  // d0 shift -1
              int hi_c = a1;
              b1 = w.pstart[rowbase];
              len1 = w.pstart[rowbase + hi_c + 1] - b1;
              sh1 = code_yz + 1;
            } else if (a1 >= P.n[0]) {
              b0 = w.pstart[rowbase + a0];
              len0 = w.pstart[rowbase + P.n[0]] - b0;
              sh0 = code_yz + 1;
              int hi_c = a1 - P.n[0];
              b1 = w.pstart[rowbase];
              len1 = w.pstart[rowbase + hi_c + 1] - b1;
              sh1 = code_yz + 2;  // d0 shift +1
            } else {
              b0 = w.pstart[rowbase + a0];
              len0 = w.pstart[rowbase + a1 + 1] - b0;
              sh0 = code_yz + 1;
            }
          }
        }
        seg_begin[2 * rr] = b0;
        seg_begin[2 * rr + 1] = b1;
        seg_shift[2 * rr] = sh0;
        seg_shift[2 * rr + 1] = sh1;
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
      int seg = 0;
      // two-entry cache of this thread's partial sums, keyed by histogram index
      int ck0 = -1, ck1 = -1;
      unsigned cn0 = 0, cn1 = 0;
      long long cd0 = 0, cp0 = 0, cx0 = 0, cd1 = 0, cp1 = 0, cx1 = 0;
      for (int t = tid; t < total; t += blockDim.x) {
        while (t >= seg_pref[seg + 1]) ++seg;
        const int pidx = seg_begin[seg] + (t - seg_pref[seg]);
        const int plab = w.plab_s[pidx];
        const int slot = slot_of[plab];
        const int base = slot * nb;
        if (MIXED) {
          const float4* A = reinterpret_cast<const float4*>(smem + SL.shapes);
          const float4* B = A + P.shapes_per_unit;
          const float2* C = reinterpret_cast<const float2*>(B + P.shapes_per_unit);
          const int* I = reinterpret_cast<const int*>(C + P.shapes_per_unit);
          float pxh = w.pxh[pidx], pxl = w.pxl[pidx];
          float pyh = w.pyh[pidx], pyl = w.pyl[pidx];
          float pzh = w.pzh[pidx], pzl = w.pzl[pidx];
          const float pw = w.pwf[pidx];
          const int code = seg_shift[seg];
          shift_hilo(pxh, pxl, code % 3 - 1, P.Lf_hi, P.Lf_lo);
          shift_hilo(pyh, pyl, (code / 3) % 3 - 1, P.Lf_hi, P.Lf_lo);
          shift_hilo(pzh, pzl, code / 9 - 1, P.Lf_hi, P.Lf_lo);
          for (int i = 0; i < S; ++i) {
            const float4 a = A[i];
            const float4 b = B[i];
            float dz = (a.z - pzh) + (b.z - pzl);
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
            if (KIND == MIA_KIND_W && fabsf(dz) > P.los_cut) continue;
            float dx = (a.x - pxh) + (b.x - pxl);
            float dy = (a.y - pyh) + (b.y - pyl);
            if (FULL) {
              // pairs whose nearest image differs from the cell image: FP64 decides
              if (P.full[0] && fabsf(dx) >= P.halfLf - P.wrap_guard) edge = true;
              if (P.full[1] && fabsf(dy) >= P.halfLf - P.wrap_guard) edge = true;
            }
            const float qp = fmaf(dx, dx, dy * dy);
            const float q = KIND == MIA_KIND_W ? qp : fmaf(dz, dz, qp);
            // early rejection: surely beyond the last binned separation
            if (q > P.q_cut) continue;
            // r bin: logarithmic bucket of q, exact FP64 breakpoints with a guard band
            int iv;
            {
              int bucket = (int)(__float_as_uint(q) >> (23 - kLutMantBits)) - P.lut32_base;
              unsigned short e;
              if (bucket >= 0 && bucket < kLut) e = T.lut32[bucket];
              else e = 0x8000;
              iv = e & 0x7fff;
              if (e & 0x8000) {
                while (iv < P.n_qbreak && q >= T.q_hi32[iv]) ++iv;
                if (iv < P.n_qbreak && q >= T.q_lo32[iv]) edge = true;
              }
            }
            const int ib = T.q_bin[iv];
            if (ib < 0 && !edge) continue;
            int jb;
            {
              float v;
              if (KIND == MIA_KIND_W) {
                v = dz;
              } else {
                if (P.rp_cut2 == 0.0) {
                  if (!(qp > 0.0f) && !edge) continue;  // r_p > rp_cut = 0 (measure_m_box_jk.py:637)
                } else {
                  const float rc2 = (float)P.rp_cut2;
                  if (qp < rc2 * (1.0f - 1e-5f)) { if (!edge) continue; }
                  else if (qp <= rc2 * (1.0f + 1e-5f)) edge = true;
                }
                v = dz * rsqrtf(q);
              }
              float t2 = (v - P.p_lo32) * P.p_inv32;
              float fl = floorf(t2);
              float fr = t2 - fl;
              jb = (int)fl;
              if (fr < P.p_guard || fr > 1.0f - P.p_guard) edge = true;
              if (jb < 0 || jb >= P.n_p) jb = -1;
            }
            if (!edge && jb < 0) continue;
            const float cx = C[i].x, cy = C[i].y;
            const float dot = fmaf(dx, cx, dy * cy);
            const float crs = fmaf(dx, cy, -dy * cx);
            if (crs * crs < P.c_guard * qp) edge = true;
            if (edge) {
              unsigned long long k = atomicAdd(&w.status->edge_count, 1ULL);
              if (k < (unsigned long long)P.edge_capacity) w.edges[k] = make_int2(I[i], pidx);
              else atomicOr(&w.status->flags, kStatusOverflow);
              continue;
            }
            const int bin = ib * P.n_p + jb;
            const float inv = __fdividef(1.0f, qp);
            const float cos2 = (dot * dot - crs * crs) * inv;
            const float sin2 = 2.0f * dot * fabsf(crs) * inv;
            const float ww = pw * a.w;
            const float we = pw * b.w;
            ++my_binned;
            if (slot >= 0) {
              const int hi = base + bin;
              const int vd = __float2int_rn(ww * fixed_scale);
              const int vp = __float2int_rn(we * cos2 * fixed_scale);
              const int vx = __float2int_rn(we * sin2 * fixed_scale);
              if (VAR || !MIA_BIN_CACHE) {
                atomicAdd(&h_cnt[hi], 1u);
                acc_fixed(dd_lo, dd_hi, hi, vd);
                acc_fixed(sp_lo, sp_hi, hi, vp);
                acc_fixed(sx_lo, sx_hi, hi, vx);
                if (VAR) {
                  float tv = we * cos2 / (float)twoR;
                  acc_fixed(vr_lo, vr_hi, hi, __float2int_rn(tv * tv * fixed_scale));
                }
              } else if (hi == ck0) {
                ++cn0; cd0 += vd; cp0 += vp; cx0 += vx;
              } else if (hi == ck1) {  // hit in the older entry: make it the newer one
                const int tk = ck0; const unsigned tn = cn0; const long long td = cd0, tp = cp0, tx = cx0;
                ck0 = ck1; cn0 = cn1 + 1; cd0 = cd1 + vd; cp0 = cp1 + vp; cx0 = cx1 + vx;
                ck1 = tk; cn1 = tn; cd1 = td; cp1 = tp; cx1 = tx;
              } else {  // miss: evict the older entry to shared memory
                if (ck1 >= 0) {
                  atomicAdd(&h_cnt[ck1], cn1);
                  add64_shared(dd_lo, dd_hi, ck1, cd1);
                  add64_shared(sp_lo, sp_hi, ck1, cp1);
                  add64_shared(sx_lo, sx_hi, ck1, cx1);
                }
                ck1 = ck0; cn1 = cn0; cd1 = cd0; cp1 = cp0; cx1 = cx0;
                ck0 = hi; cn0 = 1; cd0 = vd; cp0 = vp; cx0 = vx;
              }
            } else {
              double sp = (double)(we * cos2);
              double tv = sp / twoR;
              acc_global(o, nb, P.J, u.label, plab, bin, (double)ww, sp, (double)(we * sin2), tv * tv, VAR);
              atomicOr(&w.status->flags, kStatusNoSlot);
            }
          }
        } else {
          const double* D = reinterpret_cast<const double*>(smem + SL.shapes);
          const int M = P.shapes_per_unit;
          const double qx = w.px[pidx], qy = w.py[pidx], qz = w.pz[pidx], pw = w.pw[pidx];
          for (int i = 0; i < S; ++i) {
            PairResult r = pair_exact(P, *w.tables, D[i], D[M + i], D[2 * M + i], D[3 * M + i], D[4 * M + i],
                                      D[5 * M + i], qx, qy, qz);
            if (r.bin < 0) continue;
            const double ww = __dmul_rn(pw, D[6 * M + i]);
            const double sp = __dmul_rn(ww, r.ep);
            const double sx = __dmul_rn(ww, r.ex);
            ++my_binned;
            double tv = 0.0;
            if (VAR) tv = __ddiv_rn(sp, twoR);
            if (slot >= 0) {
              const int hi = base + r.bin;
              atomicAdd(&h_cnt[hi], 1u);
              atomicAdd(&dd_d[hi], ww);
              atomicAdd(&sp_d[hi], sp);
              atomicAdd(&sx_d[hi], sx);
              if (VAR) atomicAdd(&vr_d[hi], __dmul_rn(tv, tv));
            } else {
              acc_global(o, nb, P.J, u.label, plab, r.bin, ww, sp, sx, __dmul_rn(tv, tv), VAR);
              atomicOr(&w.status->flags, kStatusNoSlot);
            }
          }
        }
      }
      if (MIXED && !VAR && MIA_BIN_CACHE) {
        if (ck0 >= 0) {
          atomicAdd(&h_cnt[ck0], cn0);
          add64_shared(dd_lo, dd_hi, ck0, cd0);
          add64_shared(sp_lo, sp_hi, ck0, cp0);
          add64_shared(sx_lo, sx_hi, ck0, cx0);
        }
        if (ck1 >= 0) {
          atomicAdd(&h_cnt[ck1], cn1);
          add64_shared(dd_lo, dd_hi, ck1, cd1);
          add64_shared(sp_lo, sp_hi, ck1, cp1);
          add64_shared(sx_lo, sx_hi, ck1, cx1);
        }
      }
      __syncthreads();
    }

    // -- flush the unit's histograms
    const int ns = s_nslots;
    const int a = u.label;
    for (int idx = tid; idx < ns * nb; idx += blockDim.x) {
      const int k = idx / nb, bin = idx - k * nb;
      const unsigned cnt = h_cnt[idx];
      if (cnt == 0) continue;
      double dd, sp, sx, vr = 0.0;
      if (MIXED) {
        dd = fixed_value(dd_lo, dd_hi, idx, fixed_inv);
        sp = fixed_value(sp_lo, sp_hi, idx, fixed_inv);
        sx = fixed_value(sx_lo, sx_hi, idx, fixed_inv);
        if (VAR) vr = fixed_value(vr_lo, vr_hi, idx, fixed_inv);
      } else {
        dd = dd_d[idx];
        sp = sp_d[idx];
        sx = sx_d[idx];
        if (VAR) vr = vr_d[idx];
      }
      const int b = slot_region[k];
      atomicAdd(&o.npairs[bin], (unsigned long long)cnt);
      atomicAdd(&o.dd[bin], dd);
      atomicAdd(&o.splus[bin], sp);
      atomicAdd(&o.scross[bin], sx);
      if (VAR) atomicAdd(&o.variance[bin], vr);
      if (P.J > 0) {
        size_t ia = (size_t)(1 + a) * nb + bin;
        atomicAdd(&o.npairs[ia], (unsigned long long)cnt);
        atomicAdd(&o.dd[ia], dd);
        atomicAdd(&o.splus[ia], sp);
        if (b != a) {
          size_t ibb = (size_t)(1 + b) * nb + bin;
          atomicAdd(&o.npairs[ibb], (unsigned long long)cnt);
          atomicAdd(&o.dd[ibb], dd);
          atomicAdd(&o.splus[ibb], sp);
        }
      }
    }
    __syncthreads();
  }
  // binned-pair total for the throughput figure
  for (int of = 16; of > 0; of >>= 1) my_binned += __shfl_down_sync(0xffffffffu, my_binned, of);
  if ((tid & 31) == 0 && my_binned) atomicAdd(&w.status->binned, my_binned);
}

// FP64 re-test of the pairs the mixed kernel could not decide in FP32.
__global__ void k_edge_retest(Params P, Work w, Out o) {
  const unsigned long long n_raw = w.status->edge_count;
  const unsigned long long n = n_raw < (unsigned long long)P.edge_capacity ? n_raw : (unsigned long long)P.edge_capacity;
  const double twoR = 2.0 * (w.reg.s1[P.J] / w.reg.s2[P.J]);
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
    acc_global(o, P.nb, P.J, w.slab_s[si], w.plab_s[pi], r.bin, ww, sp, sx, __dmul_rn(tv, tv), P.want_variance);
    ++binned;
  }
  for (int of = 16; of > 0; of >>= 1) binned += __shfl_down_sync(0xffffffffu, binned, of);
  if ((threadIdx.x & 31) == 0 && binned) atomicAdd(&w.status->binned, binned);
}

template <int MIXED, int VAR, int KIND, int FULL>
cudaError_t launch_one(const Params& P, const Work& w, const Out& o, cudaStream_t st, int num_sms, int K) {
  SmemLayout SL = smem_layout(P.J, P.shapes_per_unit, K, P.nb, MIXED, VAR);
  size_t smem = SL.total;
  auto kern = k_pairs<MIXED, VAR, KIND, FULL>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  kern<<<num_sms * per_sm, kThreads, smem, st>>>(P, w, o, K);
  return cudaGetLastError();
}

template <int MIXED, int VAR>
cudaError_t launch_kind(const Params& P, const Work& w, const Out& o, cudaStream_t st, int num_sms, int K) {
  const bool full = P.full[0] || P.full[1] || P.full[2];
  if (P.kind == MIA_KIND_W)
    return full ? launch_one<MIXED, VAR, MIA_KIND_W, 1>(P, w, o, st, num_sms, K)
                : launch_one<MIXED, VAR, MIA_KIND_W, 0>(P, w, o, st, num_sms, K);
  return full ? launch_one<MIXED, VAR, MIA_KIND_MULTIPOLES, 1>(P, w, o, st, num_sms, K)
              : launch_one<MIXED, VAR, MIA_KIND_MULTIPOLES, 0>(P, w, o, st, num_sms, K);
}

}  // namespace

size_t pair_smem_bytes(int J, int spu, int K, int nb, int mixed, int var) {
  return smem_layout(J, spu, K, nb, mixed, var).total;
}

cudaError_t launch_pairs(const Plan& plan, const Params& P, const Work& w, const Out& o, cudaStream_t st,
                         int num_sms) {
  // slots: as many regions as a neighbourhood can touch, within the shared-memory budget
  int K = plan.J > 0 ? kMaxSlots : 1;
  {
    int need = 1;
    if (plan.J > 0) {
      need = 1;
      for (int k = 0; k < 3; ++k) {
        int span = plan.full[k] ? plan.n[k] : 2 * plan.R[k] + 1;
        int per_sub = plan.n[k] / plan.n_sub;
        int m = (span + per_sub - 1) / per_sub + 1;
        if (m > plan.n_sub) m = plan.n_sub;
        need *= m;
      }
      need += 1;
    }
    if (need < K) K = need;
    const size_t budget = 200 * 1024;
    while (K > 1 && pair_smem_bytes(plan.J, P.shapes_per_unit, K, P.nb, P.precision == MIA_MIXED, P.want_variance) >
                        budget)
      --K;
  }
  cudaError_t e;
  if (P.precision == MIA_MIXED) {
    e = P.want_variance ? launch_kind<1, 1>(P, w, o, st, num_sms, K) : launch_kind<1, 0>(P, w, o, st, num_sms, K);
    if (e != cudaSuccess) return e;
    k_edge_retest<<<num_sms * 4, 256, 0, st>>>(P, w, o);
    e = cudaGetLastError();
  } else {
    e = P.want_variance ? launch_kind<0, 1>(P, w, o, st, num_sms, K) : launch_kind<0, 0>(P, w, o, st, num_sms, K);
  }
  return e;
}

}  // namespace mia
