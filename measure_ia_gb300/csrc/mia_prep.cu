// Preparation stage: per-galaxy quantities, jackknife labels, counting sort of
// both samples into the periodic cell grid, and the work-unit list.
//
// Reference steps covered:
//   axis normalisation and e(q)          measure_w_box_jk.py:688-690, 737-742
//   responsivity sums R, R_jk            measure_w_box_jk.py:744, 782-785
//   jackknife sub-box labels             measure_IA_base.py:404-452
//   per-region galaxy counts for RR_jk   measure_w_box_jk.py:800-802
// The KD-tree build (measure_w_box_jk.py:764) is replaced by the cell list.
#include <cstdio>

#include "mia_internal.cuh"

namespace mia {

namespace {

struct PrepArgs {
  double L;
  double L_sub;      // L_0p5 * 2.0 / L_subboxes, as the reference forms it
  double inv_L_sub;  // 1 / L_sub: a first guess of the sub-box index only
  int n_sub, J;
  int axis[3];       // original axis of cell dimension k
  int n[3];
  double inv_s[3];
  int nf[3];          // position (fine) grid
  double inv_sf[3];
  int ellipticity;
};

// Jackknife label of a point (original axes): i*n^2 + j*n + k for the sub-box
// it lies strictly inside, 0 on any face or outside (measure_IA_base.py:428-451).
// x * (1 / L_sub) guesses the index to within one (no FP64 division, slow on
// this part); the exact products k * L_sub, as the reference forms its bounds,
// then move it to the sub-box that strictly contains x, if any.
__device__ __forceinline__ int jk_label(const double v[3], double L_sub, double inv_L_sub, int n_sub) {
  if (n_sub <= 1) return 0;
  int idx[3];
  for (int a = 0; a < 3; ++a) {
    double x = v[a];
    int k = (int)floor(x * inv_L_sub);
    k = k < 0 ? 0 : (k >= n_sub ? n_sub - 1 : k);
    double lo = __dmul_rn((double)k, L_sub);
    double hi = __dmul_rn((double)(k + 1), L_sub);
    if (!(x > lo) && k > 0) {
      --k;
      hi = lo;
      lo = __dmul_rn((double)k, L_sub);
    } else if (!(x < hi) && k < n_sub - 1) {
      ++k;
      lo = hi;
      hi = __dmul_rn((double)(k + 1), L_sub);
    }
    if (!(x > lo && x < hi)) return 0;
    idx[a] = k;
  }
  return (idx[0] * n_sub + idx[1]) * n_sub + idx[2];
}

__device__ __forceinline__ bool in_box(double x, double L) { return x >= 0.0 && x < L; }

__device__ __forceinline__ void flag_range(Status* st, long long i) {
  atomicOr(&st->flags, kStatusRange);
  atomicMin(&st->bad_index, (unsigned long long)i);
}

__device__ __forceinline__ int cell_of(const double c[3], const PrepArgs& A, int ci[3]) {
  for (int k = 0; k < 3; ++k) {
    int v = (int)floor(c[k] * A.inv_s[k]);
    v = v < 0 ? 0 : (v >= A.n[k] ? A.n[k] - 1 : v);
    ci[k] = v;
  }
  return (ci[2] * A.n[1] + ci[1]) * A.n[0] + ci[0];
}

__device__ __forceinline__ int fine_cell_of(const double c[3], const PrepArgs& A) {
  int ci[3];
  for (int k = 0; k < 3; ++k) {
    int v = (int)floor(c[k] * A.inv_sf[k]);
    ci[k] = v < 0 ? 0 : (v >= A.nf[k] ? A.nf[k] - 1 : v);
  }
  return (ci[2] * A.nf[1] + ci[1]) * A.nf[0] + ci[0];
}

// Region a cell lies in (cells refine the sub-box grid: n[k] is a multiple of n_sub).
__device__ __forceinline__ int natural_region(const int ci[3], const PrepArgs& A) {
  if (A.n_sub <= 1) return 0;
  int sub[3];
  for (int k = 0; k < 3; ++k) sub[A.axis[k]] = (int)((long long)ci[k] * A.n_sub / A.n[k]);
  return (sub[0] * A.n_sub + sub[1]) * A.n_sub + sub[2];
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x > v ? x : v;
  }
  return v;
}

// Per-galaxy labels and cells.  Region counts and sums go to per-block shared
// histograms (J entries, dynamic shared memory) flushed once per block, and
// the largest |weight| (bit pattern of a non-negative double: integer order =
// value order) to one atomic per warp: a few hundred blocks then touch the
// J + 2 global words instead of every galaxy.
__global__ void k_prep_positions(PrepArgs A, const double* __restrict__ pos, const double* __restrict__ w_in,
                                 long long n, Work w) {
  extern __shared__ __align__(8) unsigned char prep_smem[];
  unsigned* s_np = reinterpret_cast<unsigned*>(prep_smem);
  for (int j = threadIdx.x; j < A.J; j += blockDim.x) s_np[j] = 0u;
  __syncthreads();
  unsigned long long mx = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    if (!(in_box(v[0], A.L) && in_box(v[1], A.L) && in_box(v[2], A.L))) flag_range(w.status, i);
    double c[3] = {v[A.axis[0]], v[A.axis[1]], v[A.axis[2]]};
    int cell = fine_cell_of(c, A);
    int lab = jk_label(v, A.L_sub, A.inv_L_sub, A.n_sub);
    w.pcell[i] = cell;
    w.plab[i] = lab;
    atomicAdd(&w.pcount[cell], 1);
    if (A.J > 0) atomicAdd(&s_np[lab], 1u);
    const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(w_in[i]));
    mx = b > mx ? b : mx;
  }
  mx = warp_max_u64(mx);
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(&w.status->maxw_bits, mx);
  __syncthreads();
  for (int j = threadIdx.x; j < A.J; j += blockDim.x)
    if (s_np[j]) atomicAdd(&w.reg.npos[j], (unsigned long long)s_np[j]);
}

__global__ void k_prep_shapes(PrepArgs A, const double* __restrict__ spos, const double* __restrict__ q,
                              const double* __restrict__ ws, long long n, Work w) {
  extern __shared__ __align__(8) unsigned char prep_smem[];
  unsigned* s_ns = reinterpret_cast<unsigned*>(prep_smem);
  for (int j = threadIdx.x; j < A.J; j += blockDim.x) s_ns[j] = 0u;
  __syncthreads();
  unsigned long long mx = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v[3] = {spos[3 * i], spos[3 * i + 1], spos[3 * i + 2]};
    if (!(in_box(v[0], A.L) && in_box(v[1], A.L) && in_box(v[2], A.L))) flag_range(w.status, i);
    double c[3] = {v[A.axis[0]], v[A.axis[1]], v[A.axis[2]]};
    int ci[3];
    int cell = cell_of(c, A, ci);
    int lab = jk_label(v, A.L_sub, A.inv_L_sub, A.n_sub);
    w.scell[i] = cell;
    w.slab[i] = lab;
    atomicAdd(&w.scount[cell], 1);
    // e(q) and the responsivity weight w_s (1 - e^2 / 2)  (measure_w_box_jk.py:737-744)
    double qq = q[i], e;
    if (A.ellipticity == MIA_DISTORTION) {
      double q2 = __dmul_rn(qq, qq);
      e = __ddiv_rn(__dsub_rn(1.0, q2), __dadd_rn(1.0, q2));
    } else {
      e = __ddiv_rn(__dsub_rn(1.0, qq), __dadd_rn(1.0, qq));
    }
    const double wsi = ws[i];
    if (A.J > 0) atomicAdd(&s_ns[lab], 1u);
    const double mws = fmax(fabs(wsi), fabs(wsi * e));
    const unsigned long long b = (unsigned long long)__double_as_longlong(mws);
    mx = b > mx ? b : mx;
  }
  mx = warp_max_u64(mx);
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(&w.status->maxws_bits, mx);
  __syncthreads();
  for (int j = threadIdx.x; j < A.J; j += blockDim.x)
    if (s_ns[j]) atomicAdd(&w.reg.nshape[j], (unsigned long long)s_ns[j]);
}

// The responsivity sums s1 = sum w_s (1 - e^2/2) and s2 = sum w_s, per region
// and in total (measure_w_box_jk.py:744, :782-785), as exact fixed-point sums
// at region_scale: one int64 per term, per-block shared totals, then global
// totals.  Runs after k_prep_shapes has fixed the largest |w_s|.
__device__ __forceinline__ void add_region_terms(long long* s_r1, long long* s_r2, int lab, int J, long long v1,
                                                 long long v2, long long& t1, long long& t2) {
  if (J > 0) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&s_r1[lab]), (unsigned long long)v1);
    atomicAdd(reinterpret_cast<unsigned long long*>(&s_r2[lab]), (unsigned long long)v2);
  }
  t1 += v1;
  t2 += v2;
}

__global__ void k_region_sums(Work w, int J, long long n_shape) {
  const double inv = 1.0 / region_scale(w.status->maxws_bits, n_shape);
  for (int j = threadIdx.x; j <= J; j += blockDim.x) {
    w.reg.s1[j] = (double)w.reg.r1[j] * inv;
    w.reg.s2[j] = (double)w.reg.r2[j] * inv;
  }
}

__device__ __forceinline__ void split_hilo(double v, float& h, float& l) {
  h = __double2float_rn(v);
  l = __double2float_rn(v - (double)h);
}

__global__ void k_scatter_positions(PrepArgs A, const double* __restrict__ pos, const double* __restrict__ wgt,
                                    long long n, Work w, int mixed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int cell = w.pcell[i];
    int slot = w.pstart[cell] + atomicAdd(&w.pcur[cell], 1);
    double c0 = pos[3 * i + A.axis[0]], c1 = pos[3 * i + A.axis[1]], c2 = pos[3 * i + A.axis[2]];
    double wi = wgt[i];
    w.px[slot] = c0;
    w.py[slot] = c1;
    w.pz[slot] = c2;
    w.pw[slot] = wi;
    w.plab_s[slot] = w.plab[i];
    if (mixed) {
      split_hilo(c0, w.pxh[slot], w.pxl[slot]);
      split_hilo(c1, w.pyh[slot], w.pyl[slot]);
      split_hilo(c2, w.pzh[slot], w.pzl[slot]);
      w.pwf[slot] = __double2float_rn(wi);
    }
  }
}

__global__ void k_scatter_shapes(PrepArgs A, const double* __restrict__ spos, const double* __restrict__ axis,
                                 const double* __restrict__ q, const double* __restrict__ ws, long long n, Work w,
                                 int mixed) {
  extern __shared__ __align__(8) unsigned char prep_smem[];
  long long* s_r1 = reinterpret_cast<long long*>(prep_smem);
  long long* s_r2 = s_r1 + A.J;
  for (int j = threadIdx.x; j < A.J; j += blockDim.x) s_r1[j] = s_r2[j] = 0;
  __syncthreads();
  const double sr = region_scale(w.status->maxws_bits, n);
  long long t1 = 0, t2 = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int cell = w.scell[i];
    int lab = w.slab[i];
    double c[3] = {spos[3 * i + A.axis[0]], spos[3 * i + A.axis[1]], spos[3 * i + A.axis[2]]};
    int ci[3];
    cell_of(c, A, ci);
    bool regular = lab == natural_region(ci, A);
    int slot = regular ? w.sstart[cell] + atomicAdd(&w.scur_lo[cell], 1)
                       : w.sstart[cell + 1] - 1 - atomicAdd(&w.scur_hi[cell], 1);
    // axis normalisation: a / sqrt(a0^2 + a1^2)  (measure_w_box_jk.py:688-690)
    double a0 = axis[2 * i], a1 = axis[2 * i + 1];
    double nrm = __dsqrt_rn(__dadd_rn(__dmul_rn(a0, a0), __dmul_rn(a1, a1)));
    double ax = __ddiv_rn(a0, nrm), ay = __ddiv_rn(a1, nrm);
    double qq = q[i], e;
    if (A.ellipticity == MIA_DISTORTION) {
      double q2 = __dmul_rn(qq, qq);
      e = __ddiv_rn(__dsub_rn(1.0, q2), __dadd_rn(1.0, q2));
    } else {
      e = __ddiv_rn(__dsub_rn(1.0, qq), __dadd_rn(1.0, qq));
    }
    double wsi = ws[i];
    const double r1 = __dmul_rn(wsi, __dsub_rn(1.0, __dmul_rn(__dmul_rn(e, e), 0.5)));
    add_region_terms(s_r1, s_r2, lab, A.J, __double2ll_rn(r1 * sr), __double2ll_rn(wsi * sr), t1, t2);
    w.sx[slot] = c[0];
    w.sy[slot] = c[1];
    w.sz[slot] = c[2];
    w.sax[slot] = ax;
    w.say[slot] = ay;
    w.se[slot] = e;
    w.sws[slot] = wsi;
    w.slab_s[slot] = lab;
    if (mixed) {
      split_hilo(c[0], w.sxh[slot], w.sxl[slot]);
      split_hilo(c[1], w.syh[slot], w.syl[slot]);
      split_hilo(c[2], w.szh[slot], w.szl[slot]);
      w.saxf[slot] = __double2float_rn(ax);
      w.sayf[slot] = __double2float_rn(ay);
      w.swef[slot] = __double2float_rn(wsi * e);
      w.swsf[slot] = __double2float_rn(wsi);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    t1 += __shfl_down_sync(0xffffffffu, t1, o);
    t2 += __shfl_down_sync(0xffffffffu, t2, o);
  }
  typedef unsigned long long u64;
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(reinterpret_cast<u64*>(&w.reg.r1[A.J]), (u64)t1);
    atomicAdd(reinterpret_cast<u64*>(&w.reg.r2[A.J]), (u64)t2);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < A.J; j += blockDim.x) {
    atomicAdd(reinterpret_cast<u64*>(&w.reg.r1[j]), (u64)s_r1[j]);
    atomicAdd(reinterpret_cast<u64*>(&w.reg.r2[j]), (u64)s_r2[j]);
  }
}

// ---- exclusive scan over int counts (tiles of kScanTile) -------------------

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh_warp, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = lane < nw ? sh_warp[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) sh_warp[lane] = t;
  }
  __syncthreads();
  int before = wid > 0 ? sh_warp[wid - 1] : 0;
  total = sh_warp[nw - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void k_scan_reduce(const int* __restrict__ in, long long n, int* tiles) {
  long long base = (long long)blockIdx.x * kScanTile;
  int s = 0;
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
    long long i = base + k;
    if (i < n) s += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ int sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    tiles[blockIdx.x] = t;
  }
}

__global__ void k_scan_top(int* tiles, int n_tiles) {
  __shared__ int sh[32];
  int carry = 0;
  for (int base = 0; base < n_tiles; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < n_tiles ? tiles[i] : 0;
    int total;
    int ex = block_exclusive_scan(v, sh, total);
    if (i < n_tiles) tiles[i] = ex + carry;
    carry += total;
  }
}

// out[i] = exclusive prefix; out[n] = grand total (when write_total).
__global__ void k_scan_down(const int* __restrict__ in, long long n, const int* __restrict__ tiles, int* out,
                            int write_total, unsigned long long* total_dst) {
  __shared__ int sh[32];
  long long base = (long long)blockIdx.x * kScanTile;
  constexpr int per = kScanTile / 256;
  int v[per];
  int local = 0;
  for (int k = 0; k < per; ++k) {
    long long i = base + threadIdx.x * per + k;
    v[k] = i < n ? in[i] : 0;
    local += v[k];
  }
  int total;
  int ex = block_exclusive_scan(local, sh, total) + tiles[blockIdx.x];
  for (int k = 0; k < per; ++k) {
    long long i = base + threadIdx.x * per + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
  if (write_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {
    // the last thread of the last tile holds the grand total in ex
    out[n] = ex;
    if (total_dst) *total_dst = (unsigned long long)ex;
  }
}

cudaError_t scan(const int* in, long long n, int* out, int* tiles, unsigned long long* total_dst, cudaStream_t st) {
  int n_tiles = (int)((n + kScanTile - 1) / kScanTile);
  if (n_tiles == 0) n_tiles = 1;
  k_scan_reduce<<<n_tiles, 256, 0, st>>>(in, n, tiles);
  k_scan_top<<<1, 1024, 0, st>>>(tiles, n_tiles);
  k_scan_down<<<n_tiles, 256, 0, st>>>(in, n, tiles, out, 1, total_dst);
  return cudaGetLastError();
}

// ---- work units -------------------------------------------------------------

__global__ void k_wu_count(long long n_cells, int per_unit, Work w) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n_cells;
       c += (long long)gridDim.x * blockDim.x) {
    int reg = w.scur_lo[c], irr = w.scur_hi[c];
    w.wucount[c] = (reg + per_unit - 1) / per_unit + irr;
  }
}

__global__ void k_wu_emit(PrepArgs A, long long n_cells, int per_unit, Work w) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n_cells;
       c += (long long)gridDim.x * blockDim.x) {
    int reg = w.scur_lo[c], irr = w.scur_hi[c];
    int out = w.wustart[c];
    int first = w.sstart[c];
    if (reg > 0) {
      int ci[3];
      long long t = c;
      ci[0] = (int)(t % A.n[0]);
      t /= A.n[0];
      ci[1] = (int)(t % A.n[1]);
      ci[2] = (int)(t / A.n[1]);
      int lab = natural_region(ci, A);
      int k = (reg + per_unit - 1) / per_unit;
      int base = reg / k, extra = reg % k, b = first;
      for (int u = 0; u < k; ++u) {
        int cnt = base + (u < extra ? 1 : 0);
        w.wu[out++] = WorkUnit{(int)c, b, cnt, lab};
        b += cnt;
      }
    }
    for (int u = 0; u < irr; ++u) {
      int idx = first + reg + u;
      w.wu[out++] = WorkUnit{(int)c, idx, 1, w.slab_s[idx]};
    }
  }
}

int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 65535LL * 8) b = 65535LL * 8;
  return (int)b;
}

}  // namespace

cudaError_t launch_prep(const Plan& plan, const Params& P, const mia_catalog& cat, const Work& w, cudaStream_t st) {
  PrepArgs A;
  A.L = P.L;
  A.n_sub = plan.n_sub;
  A.L_sub = (P.L / 2.0) * 2.0 / (double)(plan.n_sub > 0 ? plan.n_sub : 1);
  A.inv_L_sub = 1.0 / A.L_sub;
  A.J = plan.J;
  for (int k = 0; k < 3; ++k) {
    A.axis[k] = plan.axis[k];
    A.n[k] = plan.n[k];
    A.inv_s[k] = (double)plan.n[k] / P.L;
    A.nf[k] = plan.nf[k];
    A.inv_sf[k] = (double)plan.nf[k] / P.L;
  }
  A.ellipticity = P.ellipticity;
  const int T = 256;
  int mixed = P.precision == MIA_MIXED;
  // at most 1024 blocks, so that the per-block region histograms are flushed
  // a bounded number of times
  const int gp = grid_for(cat.n_pos, T) < 1024 ? grid_for(cat.n_pos, T) : 1024;
  const int gs = grid_for(cat.n_shape, T) < 1024 ? grid_for(cat.n_shape, T) : 1024;
  k_prep_positions<<<gp, T, sizeof(unsigned) * (size_t)plan.J, st>>>(A, cat.position, cat.weight, cat.n_pos, w);
  k_prep_shapes<<<gs, T, sizeof(unsigned) * (size_t)plan.J, st>>>(
      A, cat.position_shape, cat.q, cat.weight_shape, cat.n_shape, w);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = scan(w.pcount, plan.n_fcells, w.pstart, w.tiles, nullptr, st)) != cudaSuccess) return e;
  if ((e = scan(w.scount, plan.n_cells, w.sstart, w.tiles, nullptr, st)) != cudaSuccess) return e;
  k_scatter_positions<<<grid_for(cat.n_pos, T), T, 0, st>>>(A, cat.position, cat.weight, cat.n_pos, w, mixed);
  k_scatter_shapes<<<gs, T, 2 * sizeof(long long) * (size_t)plan.J, st>>>(
      A, cat.position_shape, cat.axis_direction, cat.q, cat.weight_shape, cat.n_shape, w, mixed);
  k_region_sums<<<1, 256, 0, st>>>(w, plan.J, cat.n_shape);
  k_wu_count<<<grid_for(plan.n_cells, T), T, 0, st>>>(plan.n_cells, plan.shapes_per_unit, w);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = scan(w.wucount, plan.n_cells, w.wustart, w.tiles, &w.status->n_wu, st)) != cudaSuccess) return e;
  k_wu_emit<<<grid_for(plan.n_cells, T), T, 0, st>>>(A, plan.n_cells, plan.shapes_per_unit, w);
  return cudaGetLastError();
}

cudaError_t exclusive_scan(const int* in, long long n, int* out, int* tiles, cudaStream_t st) {
  return scan(in, n, out, tiles, nullptr, st);
}

}  // namespace mia
