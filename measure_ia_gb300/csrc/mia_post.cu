// Post-processing on the device, all FP64: responsivities, analytic randoms,
// correlation functions of the full sample and of every jackknife
// realisation, Pi integration (w) or Legendre multipoles, and the jackknife
// mean / standard deviation / covariance.
//
// Reference formulas (measure_IA_base.py unless noted):
//   R, R_jk                 measure_w_box_jk.py:744, 782-785
//   RR (r_p, Pi)            get_random_pairs, 'cross'          :268-269
//   RR (r, mu_r)            get_random_pairs_r_mur, 'cross'    :293-351
//   RR_jk volumes           measure_w_box_jk.py:798-807
//   realisations            measure_w_box_jk.py:825-853
//   w = sum xi |dpi|        _measure_w_g_i                     :547-562
//   multipoles              _measure_multipoles                :628-655
//   mean / std / cov        _combine_jackknife_information     :481-498
// Operand order follows the reference's expressions so that the products
// agree with it to a few ulps.
#include "mia_internal.cuh"

namespace mia {

namespace {

struct PostArgs {
  int kind, J, n_r, n_p, nb, want_variance;
  double volume;
  long long n_pos, n_shape;
};

__device__ __forceinline__ double cap_volume(double mur, double r) {
  // np.pi / 3.0 * r ** 3 * (2 + mur) * (1 - mur) ** 2
  const double pi3 = 3.141592653589793 / 3.0;
  double om = __dsub_rn(1.0, mur);
  return __dmul_rn(__dmul_rn(__dmul_rn(pi3, __dmul_rn(__dmul_rn(r, r), r)), __dadd_rn(2.0, mur)), __dmul_rn(om, om));
}

__device__ double rr_bin(const PostArgs& A, const Tables& T, int i, int p, double vol, double np_, double ns_) {
  const double pi = 3.141592653589793;
  double rhi = T.r_edges[i + 1], rlo = T.r_edges[i];
  double phi = T.p_edges[p + 1], plo = T.p_edges[p];
  if (A.kind == MIA_KIND_W) {
    // Num_position * Num_shape * np.pi * (rp_max**2 - rp_min**2) * abs(pi_max - pi_min) / L3
    double d2 = __dsub_rn(__dmul_rn(rhi, rhi), __dmul_rn(rlo, rlo));
    double v = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(np_, ns_), pi), d2), fabs(__dsub_rn(phi, plo)));
    return __ddiv_rn(v, vol);
  }
  // (Num_position - 1.0) * Num_shape * (V(mu_min, r_max) - V(mu_max, r_max) - (V(mu_min, r_min) - V(mu_max, r_min))) / L3
  double big = __dsub_rn(cap_volume(plo, rhi), cap_volume(phi, rhi));
  double small = __dsub_rn(cap_volume(plo, rlo), cap_volume(phi, rlo));
  double v = __dmul_rn(__dmul_rn(__dsub_rn(np_, 1.0), ns_), __dsub_rn(big, small));
  return fabs(__ddiv_rn(v, vol));
}

// w (Pi integration) or the multipole of one xi grid row.
__device__ double project_row(const PostArgs& A, const Tables& T, const double* xi_row, int l) {
  double acc = 0.0;
  if (A.kind == MIA_KIND_W) {
    for (int p = 0; p < A.n_p; ++p) acc += xi_row[p] * fabs(T.p_edges[p + 1] - T.p_edges[p]);
    return acc;
  }
  // (2l+1)/2 * (l-m)!/(l+m)! * P_l^m(mu_c) * xi * dmu, m = l; P_2^2 = 3 (1 - mu^2), P_0^0 = 1
  double fac = l == 2 ? (5.0 / 2.0) * 1.0 / 24.0 : (1.0 / 2.0);
  for (int p = 0; p < A.n_p; ++p) {
    double lo = T.p_edges[p], hi = T.p_edges[p + 1];
    double mu = lo + fabs((hi - lo) / 2.0);
    double P = l == 2 ? 3.0 * (1.0 - mu * mu) : 1.0;
    acc += fac * P * xi_row[p] * (hi - lo);
  }
  return acc;
}

__global__ void k_post(PostArgs A, Work w, mia_layout lay, double* out) {
  const Tables& T = *w.tables;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int J = A.J, nb = A.nb, nr = A.n_r, np = A.n_p;
  double* o = out;
  const double S1 = w.reg.s1[J], S2 = w.reg.s2[J];
  const double R = S1 / S2;
  if (tid == 0) {
    o[lay.R] = R;
    double* st = o + lay.stats;
    st[0] = (double)A.n_pos;
    st[1] = (double)A.n_shape;
    st[2] = (double)w.status->binned;
    st[3] = (double)w.status->edge_count;
    st[4] = (double)w.status->n_wu;
  }
  for (int i = tid; i < J; i += nt) {
    o[lay.R_jk + i] = (S1 - w.reg.s1[i]) / (S2 - w.reg.s2[i]);
    o[lay.npos_jk + i] = (double)(A.n_pos - (long long)w.reg.npos[i]);
    o[lay.nshape_jk + i] = (double)(A.n_shape - (long long)w.reg.nshape[i]);
  }
  // analytic randoms
  const double npd = (double)A.n_pos, nsd = (double)A.n_shape;
  for (int k = tid; k < nb; k += nt) {
    int i = k / np, p = k - i * np;
    double nps = A.kind == MIA_KIND_W ? (double)(A.n_pos * A.n_shape) : npd;
    o[lay.rr + k] = rr_bin(A, T, i, p, A.volume, nps, A.kind == MIA_KIND_W ? 1.0 : nsd);
  }
  const double vol_jk = J > 0 ? (A.volume * (double)(J - 1)) / (double)J : 0.0;
  for (int k = tid; k < J * nb; k += nt) {
    int jk = k / nb, b = k - jk * nb;
    int i = b / np, p = b - i * np;
    long long npj = A.n_pos - (long long)w.reg.npos[jk];
    long long nsj = A.n_shape - (long long)w.reg.nshape[jk];
    double nps = A.kind == MIA_KIND_W ? (double)(npj * nsj) : (double)npj;
    o[lay.rr_jk + k] = rr_bin(A, T, i, p, vol_jk, nps, A.kind == MIA_KIND_W ? 1.0 : (double)nsj);
  }
  __syncthreads();
  // full-sample products
  const double twoR = 2.0 * R;
  for (int k = tid; k < nb; k += nt) {
    double rr = o[lay.rr + k];
    double spd = o[lay.splus + k] / twoR;
    double sxd = o[lay.scross + k] / twoR;
    o[lay.splusd + k] = spd;
    o[lay.scrossd + k] = sxd;
    o[lay.xi_gp + k] = spd / rr;
    o[lay.xi_gx + k] = sxd / rr;
    o[lay.xi_gg + k] = o[lay.dd + k] / rr - 1.0;
    o[lay.sigmasq + k] = A.want_variance ? o[lay.variance + k] / (rr * rr) : 0.0;
  }
  __syncthreads();
  // realisations
  for (int k = tid; k < J * nb; k += nt) {
    int i = k / nb, b = k - i * nb;
    double rrj = o[lay.rr_jk + k];
    double Rj = o[lay.R_jk + i];
    double num = o[lay.splusd + b] * twoR - o[lay.splus + (size_t)(1 + i) * nb + b];
    o[lay.xi_gp_jk + k] = num / (rrj * 2.0 * Rj);
    o[lay.splusd_jk + k] = num / (2.0 * Rj);
    double ddi = o[lay.dd + b] - o[lay.dd + (size_t)(1 + i) * nb + b];
    o[lay.dd_jk + k] = ddi;
    o[lay.xi_gg_jk + k] = ddi / rrj - 1.0;
  }
  __syncthreads();
  // projections: full sample and realisations
  for (int k = tid; k < (1 + J) * nr; k += nt) {
    int i = k / nr, r = k - i * nr;
    if (i == 0) {
      o[lay.proj_gp + r] = project_row(A, T, o + lay.xi_gp + (size_t)r * np, 2);
      o[lay.proj_gg + r] = project_row(A, T, o + lay.xi_gg + (size_t)r * np, 0);
    } else {
      size_t row = (size_t)(i - 1) * nb + (size_t)r * np;
      o[lay.proj_gp_jk + (size_t)(i - 1) * nr + r] = project_row(A, T, o + lay.xi_gp_jk + row, 2);
      o[lay.proj_gg_jk + (size_t)(i - 1) * nr + r] = project_row(A, T, o + lay.xi_gg_jk + row, 0);
    }
  }
  __syncthreads();
  if (J == 0) return;
  // jackknife mean, std and covariance over the realisations
  const double f = (double)(J - 1) / (double)J;
  for (int which = 0; which < 2; ++which) {
    const double* x = o + (which == 0 ? lay.proj_gp_jk : lay.proj_gg_jk);
    double* mean = o + (which == 0 ? lay.mean_gp : lay.mean_gg);
    double* sd = o + (which == 0 ? lay.std_gp : lay.std_gg);
    double* cov = o + (which == 0 ? lay.cov_gp : lay.cov_gg);
    for (int r = tid; r < nr; r += nt) {
      double m = 0.0;
      for (int b = 0; b < J; ++b) m += x[(size_t)b * nr + r];
      mean[r] = m / (double)J;
    }
    __syncthreads();
    for (int r = tid; r < nr; r += nt) {
      double s = 0.0;
      for (int b = 0; b < J; ++b) {
        double d = x[(size_t)b * nr + r] - mean[r];
        s += d * d;
      }
      sd[r] = sqrt(s * f);
    }
    for (int k = tid; k < nr * nr; k += nt) {
      int a = k / nr, c = k - a * nr;  // cov[a][c]
      double s = 0.0;
      for (int b = 0; b < J; ++b) s += (x[(size_t)b * nr + a] - mean[a]) * (x[(size_t)b * nr + c] - mean[c]);
      cov[k] = s * f;
    }
    __syncthreads();
  }
}

// Jackknife covariance of two datasets' realisations (measure_jackknife.py:
// 519-555): realisation means, cov[j][i] = f * sum_r (a_r[j] - ma[j]) *
// (b_r[i] - mb[i]) and std[j] = sqrt(f * sum_r (a_r[j] - ma[j]) *
// (b_r[j] - mb[j])), f = (n - 1) / n, every sum in realisation order and
// every product rounded before its add, as numpy forms them.  A block owns a
// 32 x 32 tile of cov (rows j, columns i) and first forms the means of its 32
// a-columns and 32 b-columns; the tiles on the diagonal also write std.
constexpr int kCovTile = 32;

__global__ void k_cross_cov(int n_real, int n_bins, const double* __restrict__ a, long long sa,
                            const double* __restrict__ b, long long sb, double* cov, double* std) {
  __shared__ double ma[kCovTile], mb[kCovTile];
  const int j0 = blockIdx.y * kCovTile, i0 = blockIdx.x * kCovTile;
  const int t = threadIdx.x;
  if (t < 2 * kCovTile) {
    const bool rows = t < kCovTile;
    const int col = (rows ? j0 : i0) + (t & (kCovTile - 1));
    double s = 0.0;
    if (col < n_bins) {
      const double* x = rows ? a : b;
      const long long sx = rows ? sa : sb;
      for (int r = 0; r < n_real; ++r) s = __dadd_rn(s, x[r * sx + col]);
      s = __ddiv_rn(s, (double)n_real);
    }
    (rows ? ma : mb)[t & (kCovTile - 1)] = s;
  }
  __syncthreads();
  const double f = __ddiv_rn((double)(n_real - 1), (double)n_real);
  const int ti = t & (kCovTile - 1);
  const int i = i0 + ti;
  for (int tj = t / kCovTile; tj < kCovTile; tj += blockDim.x / kCovTile) {
    const int j = j0 + tj;
    if (j >= n_bins || i >= n_bins) continue;
    double s = 0.0;
    for (int r = 0; r < n_real; ++r)
      s = __dadd_rn(s, __dmul_rn(__dsub_rn(a[r * sa + j], ma[tj]), __dsub_rn(b[r * sb + i], mb[ti])));
    const double v = __dmul_rn(s, f);
    cov[(long long)j * n_bins + i] = v;
    if (i == j) std[j] = __dsqrt_rn(v);
  }
}

}  // namespace

cudaError_t launch_cross_cov(int n_real, int n_bins, const double* a, long long sa, const double* b, long long sb,
                             double* cov, double* std, cudaStream_t st) {
  const int tiles = (n_bins + kCovTile - 1) / kCovTile;
  k_cross_cov<<<dim3(tiles, tiles), 256, 0, st>>>(n_real, n_bins, a, sa, b, sb, cov, std);
  return cudaGetLastError();
}

cudaError_t launch_post(const Params& P, const Work& w, const mia_layout& lay, double* out, double volume,
                        long long n_pos, long long n_shape, cudaStream_t st) {
  PostArgs A;
  A.kind = P.kind;
  A.J = P.J;
  A.n_r = P.n_r;
  A.n_p = P.n_p;
  A.nb = P.nb;
  A.want_variance = P.want_variance;
  A.volume = volume;
  A.n_pos = n_pos;
  A.n_shape = n_shape;
  k_post<<<1, 256, 0, st>>>(A, w, lay, out);
  return cudaGetLastError();
}

}  // namespace mia
