// C ABI: context, sizing helpers and the mia_measure driver that enqueues the
// preparation, pair and post-processing stages.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "mia_internal.cuh"

// NVTX ranges around the enqueue of each stage (prep, pairs, re-test, post),
// so that a profiler's timeline and `ncu --nvtx --nvtx-include` can select a
// stage; they mark host enqueue time, the kernels run asynchronously.
namespace {
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

// Streams on which a batch's per-catalogue preparation (memsets, labels, cell
// list, work units: ~20 short launches each) runs side by side, forked from
// and joined back into the caller's stream with events, so that the small
// catalogues of a batch do not wait for each other.
constexpr int kPrepStreams = 4;

struct mia_context {
  int device;
  int num_sms;
  std::string err;
  // pair-kernel launch timing (mia_profile_pairs): a ring of event pairs
  std::vector<cudaEvent_t> prof_start, prof_stop;
  long long prof_count = 0;  // launches recorded since enabling
  // preparation streams and their fork / join events (created by mia_batch_prepare)
  cudaStream_t prep[kPrepStreams] = {};
  cudaEvent_t fork = nullptr, join[kPrepStreams] = {};
  bool prep_ready = false;
};

static void free_prep_streams(mia_context* c) {
  if (!c->prep_ready) return;
  for (int k = 0; k < kPrepStreams; ++k) {
    cudaStreamDestroy(c->prep[k]);
    cudaEventDestroy(c->join[k]);
  }
  cudaEventDestroy(c->fork);
  c->prep_ready = false;
}

static cudaError_t make_prep_streams(mia_context* c) {
  if (c->prep_ready) return cudaSuccess;
  cudaError_t e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
  for (int k = 0; k < kPrepStreams && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&c->prep[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join[k], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) return e;
  c->prep_ready = true;
  return cudaSuccess;
}

static void free_profile_events(mia_context* c) {
  for (cudaEvent_t e : c->prof_start) cudaEventDestroy(e);
  for (cudaEvent_t e : c->prof_stop) cudaEventDestroy(e);
  c->prof_start.clear();
  c->prof_stop.clear();
  c->prof_count = 0;
}

namespace mia {

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Bytes of a dataset's fixed-point sums: (2 (1+J) + 2) nb sums of acc_words words.
size_t acc_bytes(const Plan& p) {
  return sizeof(long long) * (size_t)p.acc_words * (size_t)p.nb * (2 * ((size_t)p.J + 1) + 2);
}

}  // namespace

bool make_plan(const mia_config* cfg, long long n_pos, long long n_shape, Plan* pl, const char** why) {
  Plan& p = *pl;
  memset(&p, 0, sizeof(p));
  if (!cfg) { *why = "null config"; return false; }
  if (cfg->kind != MIA_KIND_W && cfg->kind != MIA_KIND_MULTIPOLES) { *why = "kind"; return false; }
  if (cfg->los < 0 || cfg->los > 2) { *why = "LOS must be 0, 1 or 2"; return false; }
  if (cfg->n_r < 1 || cfg->n_r > MIA_MAX_BINS_R) { *why = "num_bins_r out of range"; return false; }
  if (cfg->n_p < 1 || cfg->n_p > MIA_MAX_BINS_P) { *why = "num_bins_pi out of range"; return false; }
  if (cfg->n_qbreak < 0 || cfg->n_qbreak > MIA_MAX_BREAKS || cfg->n_pbreak < 0 || cfg->n_pbreak > MIA_MAX_BREAKS) {
    *why = "too many breakpoints";
    return false;
  }
  if (!(cfg->boxsize > 0.0)) { *why = "boxsize must be positive"; return false; }
  if (cfg->l_subboxes < 0 || cfg->l_subboxes > 10) { *why = "jackknife sub-boxes per side must be 0..10"; return false; }
  if (n_pos < 0 || n_shape < 0 || n_pos > 0x7fffffffLL || n_shape > 0x7fffffffLL) { *why = "sample size"; return false; }
  if (!cfg->r_edges || !cfg->p_edges || !cfg->q_bin || !cfg->p_bin) { *why = "missing tables"; return false; }
  const double L = cfg->boxsize;
  p.axis[0] = cfg->los == 0 ? 1 : 0;
  p.axis[1] = cfg->los == 2 ? 1 : 2;
  p.axis[2] = cfg->los;
  p.n_sub = cfg->l_subboxes > 0 ? cfg->l_subboxes : 1;
  p.J = cfg->l_subboxes > 0 ? cfg->l_subboxes * cfg->l_subboxes * cfg->l_subboxes : 0;
  p.nb = cfg->n_r * cfg->n_p;
  double rr = fmax(cfg->r_max, cfg->r_edges[cfg->n_r]);
  p.range_proj = rr;
  if (cfg->kind == MIA_KIND_W) p.range_los = fmax(fabs(cfg->p_edges[0]), fabs(cfg->p_edges[cfg->n_p]));
  else p.range_los = rr;
  double target[3];
  double cs = cfg->cell_size > 0.0 ? cfg->cell_size : 0.0;
  target[0] = target[1] = cs > 0.0 ? cs : p.range_proj / 2.0;
  target[2] = cfg->cell_size_los > 0.0 ? cfg->cell_size_los : (cs > 0.0 ? cs : fmax(p.range_los / 2.0, 1e-300));
  long long cells = 1;
  for (int k = 0; k < 3; ++k) {
    long long n = (long long)floor(L / target[k]);
    if (n > 1024) n = 1024;
    n = (n / p.n_sub) * p.n_sub;
    if (n < p.n_sub) n = p.n_sub;
    p.n[k] = (int)n;
    cells *= n;
  }
  while (cells > (1LL << 25)) {  // keep the cell tables modest
    cells = 1;
    for (int k = 0; k < 3; ++k) {
      long long n = p.n[k] / 2;
      n = (n / p.n_sub) * p.n_sub;
      if (n < p.n_sub) n = p.n_sub;
      p.n[k] = (int)n;
      cells *= n;
    }
  }
  p.n_cells = cells;
  long long fcells = 1;
  for (int k = 0; k < 3; ++k) {
    p.s[k] = L / p.n[k];
    double range = k == 2 ? p.range_los : p.range_proj;
    long long R = (long long)ceil(range / p.s[k] * (1.0 + 1e-9));
    if (R < 1) R = 1;
    if (2 * R + 1 >= p.n[k]) R = p.n[k] / 2;
    p.R[k] = (int)R;
    // position grid: refine each shape cell m times (at most 1024 cells per side)
    int m = cfg->cell_refine > 0 ? cfg->cell_refine : 3;
    if (k == 2 && cfg->cell_refine_los > 0) m = cfg->cell_refine_los;
    while (m > 1 && (long long)m * p.n[k] > 1024) --m;
    p.m[k] = m;
    p.nf[k] = m * p.n[k];
    p.sf[k] = L / p.nf[k];
    long long Rf = (long long)ceil(range / p.sf[k] * (1.0 + 1e-9));
    if (Rf < 1) Rf = 1;
    if (m + 2 * Rf >= p.nf[k]) {
      p.full[k] = 1;
      Rf = (p.nf[k] - m + 1) / 2;
    }
    p.Rf[k] = (int)Rf;
    fcells *= p.nf[k];
  }
  // keep the position-cell tables modest: coarsen the refinement if needed
  while (fcells > (1LL << 26) && (p.m[0] > 1 || p.m[1] > 1 || p.m[2] > 1)) {
    fcells = 1;
    for (int k = 0; k < 3; ++k) {
      if (p.m[k] > 1) --p.m[k];
      p.nf[k] = p.m[k] * p.n[k];
      p.sf[k] = L / p.nf[k];
      double range = k == 2 ? p.range_los : p.range_proj;
      long long Rf = (long long)ceil(range / p.sf[k] * (1.0 + 1e-9));
      if (Rf < 1) Rf = 1;
      p.full[k] = 0;
      if (p.m[k] + 2 * Rf >= p.nf[k]) {
        p.full[k] = 1;
        Rf = (p.nf[k] - p.m[k] + 1) / 2;
      }
      p.Rf[k] = (int)Rf;
      fcells *= p.nf[k];
    }
  }
  p.n_fcells = fcells;
  p.shapes_per_unit = cfg->shapes_per_unit > 0 ? cfg->shapes_per_unit : 128;
  if (p.shapes_per_unit > kThreads) p.shapes_per_unit = kThreads;  // one staged shape per thread
  p.n_wu_max = p.n_cells + n_shape + 1;
  p.edge_capacity = 0;
  if (cfg->precision == MIA_MIXED) {
    long long cap = n_shape * 32;
    if (cap < (1LL << 20)) cap = 1LL << 20;
    if (cap > (1LL << 28)) cap = 1LL << 28;
    // MIA_EDGE_CAPACITY=<entries> replaces the default (workspace sizes follow)
    if (const char* env = std::getenv("MIA_EDGE_CAPACITY")) {
      const long long v = std::atoll(env);
      if (v > 0) cap = v;
    }
    p.edge_capacity = cap;
  }
  const bool mixed = cfg->precision == MIA_MIXED;
  size_t o = 0;
  auto take = [&](size_t& off, size_t bytes) {
    off = o;
    o = align256(o + bytes);
  };
  const size_t C = (size_t)p.n_cells;
  const size_t CF = (size_t)p.n_fcells;
  const size_t NP = (size_t)(n_pos > 0 ? n_pos : 1), NS = (size_t)(n_shape > 0 ? n_shape : 1);
  take(p.off_status, sizeof(Status));
  take(p.off_tables, sizeof(Tables));
  take(p.off_pcount, 4 * CF);
  take(p.off_pstart, 4 * (CF + 1));
  take(p.off_pcur, 4 * CF);
  take(p.off_scount, 4 * C);
  take(p.off_sstart, 4 * (C + 1));
  take(p.off_scur_lo, 4 * C);
  take(p.off_scur_hi, 4 * C);
  take(p.off_wucount, 4 * C);
  take(p.off_wustart, 4 * (C + 1));
  take(p.off_tiles, 4 * ((C > CF ? C : CF) / kScanTile + 2));
  take(p.off_pcell, 4 * NP);
  take(p.off_plab, 4 * NP);
  take(p.off_scell, 4 * NS);
  take(p.off_slab, 4 * NS);
  take(p.off_p64, 8 * 4 * NP);
  take(p.off_plab_s, 4 * NP);
  take(p.off_p32, mixed ? 4 * 7 * NP : 0);
  take(p.off_s64, 8 * 7 * NS);
  take(p.off_slab_s, 4 * NS);
  // (FP32 shape arrays 16-byte aligned each: a stride of a multiple of 4 floats)
  take(p.off_s32, mixed ? 4 * 10 * ((NS + 3) & ~size_t(3)) : 0);
  take(p.off_wu, sizeof(WorkUnit) * (size_t)p.n_wu_max);
  take(p.off_reg, (size_t)(p.J + 1) * 48 + 64);
  take(p.off_edges, sizeof(int2) * (size_t)p.edge_capacity);
  // fixed-point sums (w and S+D per region, SxD and var): one 64-bit word per
  // sum in the mixed form, two (128-bit) in the FP64 form
  p.acc_words = mixed ? 1 : 2;
  take(p.off_acc, acc_bytes(p));
  p.total = o;
  return true;
}

void bind_work(const Plan& p, void* base, Work* w) {
  unsigned char* b = static_cast<unsigned char*>(base);
  const size_t NP = 0;  // unused
  (void)NP;
  w->status = reinterpret_cast<Status*>(b + p.off_status);
  w->tables = reinterpret_cast<Tables*>(b + p.off_tables);
  w->pcount = reinterpret_cast<int*>(b + p.off_pcount);
  w->pstart = reinterpret_cast<int*>(b + p.off_pstart);
  w->pcur = reinterpret_cast<int*>(b + p.off_pcur);
  w->scount = reinterpret_cast<int*>(b + p.off_scount);
  w->sstart = reinterpret_cast<int*>(b + p.off_sstart);
  w->scur_lo = reinterpret_cast<int*>(b + p.off_scur_lo);
  w->scur_hi = reinterpret_cast<int*>(b + p.off_scur_hi);
  w->wucount = reinterpret_cast<int*>(b + p.off_wucount);
  w->wustart = reinterpret_cast<int*>(b + p.off_wustart);
  w->tiles = reinterpret_cast<int*>(b + p.off_tiles);
  w->pcell = reinterpret_cast<int*>(b + p.off_pcell);
  w->plab = reinterpret_cast<int*>(b + p.off_plab);
  w->scell = reinterpret_cast<int*>(b + p.off_scell);
  w->slab = reinterpret_cast<int*>(b + p.off_slab);
  w->plab_s = reinterpret_cast<int*>(b + p.off_plab_s);
  w->slab_s = reinterpret_cast<int*>(b + p.off_slab_s);
  w->wu = reinterpret_cast<WorkUnit*>(b + p.off_wu);
  w->edges = reinterpret_cast<int2*>(b + p.off_edges);
  unsigned char* reg = b + p.off_reg;
  const size_t J1 = (size_t)p.J + 1;
  w->reg.npos = reinterpret_cast<unsigned long long*>(reg);
  w->reg.nshape = reinterpret_cast<unsigned long long*>(reg + 8 * J1);
  w->reg.s1 = reinterpret_cast<double*>(reg + 16 * J1);
  w->reg.s2 = reinterpret_cast<double*>(reg + 24 * J1);
  w->reg.r1 = reinterpret_cast<long long*>(reg + 32 * J1);
  w->reg.r2 = reinterpret_cast<long long*>(reg + 40 * J1);
  long long* acc = reinterpret_cast<long long*>(b + p.off_acc);
  const size_t aw = (size_t)p.acc_words;
  w->acc_dd = acc;
  w->acc_sp = acc + aw * J1 * p.nb;
  w->acc_sx = acc + aw * 2 * J1 * p.nb;
  w->acc_vr = acc + aw * (2 * J1 + 1) * p.nb;
}

// Bind the per-galaxy arrays once the sample sizes are known.
static void bind_arrays(const Plan& p, void* base, long long n_pos, long long n_shape, Work* w) {
  unsigned char* b = static_cast<unsigned char*>(base);
  const size_t NP = (size_t)(n_pos > 0 ? n_pos : 1), NS = (size_t)(n_shape > 0 ? n_shape : 1);
  double* p64 = reinterpret_cast<double*>(b + p.off_p64);
  w->px = p64;
  w->py = p64 + NP;
  w->pz = p64 + 2 * NP;
  w->pw = p64 + 3 * NP;
  float* p32 = reinterpret_cast<float*>(b + p.off_p32);
  w->pxh = p32;
  w->pxl = p32 + NP;
  w->pyh = p32 + 2 * NP;
  w->pyl = p32 + 3 * NP;
  w->pzh = p32 + 4 * NP;
  w->pzl = p32 + 5 * NP;
  w->pwf = p32 + 6 * NP;
  double* s64 = reinterpret_cast<double*>(b + p.off_s64);
  w->sx = s64;
  w->sy = s64 + NS;
  w->sz = s64 + 2 * NS;
  w->sax = s64 + 3 * NS;
  w->say = s64 + 4 * NS;
  w->se = s64 + 5 * NS;
  w->sws = s64 + 6 * NS;
  float* s32 = reinterpret_cast<float*>(b + p.off_s32);
  const size_t NS4 = (NS + 3) & ~size_t(3);
  w->sxh = s32;
  w->sxl = s32 + NS4;
  w->syh = s32 + 2 * NS4;
  w->syl = s32 + 3 * NS4;
  w->szh = s32 + 4 * NS4;
  w->szl = s32 + 5 * NS4;
  w->saxf = s32 + 6 * NS4;
  w->sayf = s32 + 7 * NS4;
  w->swef = s32 + 8 * NS4;
  w->swsf = s32 + 9 * NS4;
}

static float f32_down(double v) {
  float f = (float)v;
  if ((double)f > v) f = nextafterf(f, -INFINITY);
  return f;
}
static float f32_up(double v) {
  float f = (float)v;
  if ((double)f < v) f = nextafterf(f, INFINITY);
  return f;
}

// Host-side construction of the device tables from the configuration.
static void build_tables(const mia_config* cfg, Tables* T, int* lut_base, bool* short_tables) {
  memset(T, 0, sizeof(Tables));
  const double g = 1.0 / 524288.0;  // 2^-19 relative guard band on q
  for (int j = 0; j < MIA_MAX_BREAKS; ++j) {
    if (j < cfg->n_qbreak) {
      double B = cfg->q_break[j];
      T->q_break[j] = B;
      memcpy(&T->q_key[j], &B, 8);
      T->q_lo32[j] = f32_down(B * (1.0 - g));
      T->q_hi32[j] = f32_up(B * (1.0 + g));
    } else {
      T->q_key[j] = 0x7fffffffffffffffLL;
      T->q_lo32[j] = INFINITY;
      T->q_hi32[j] = INFINITY;
    }
    if (j < cfg->n_pbreak) {
      T->p_break[j] = cfg->p_break[j];
      T->p_key[j] = order_key(cfg->p_break[j]);
    } else {
      T->p_key[j] = 0x7fffffffffffffffLL;
    }
  }
  for (int j = 0; j <= MIA_MAX_BREAKS; ++j) {
    T->q_bin[j] = j <= cfg->n_qbreak ? cfg->q_bin[j] : -1;
    T->p_bin[j] = j <= cfg->n_pbreak ? cfg->p_bin[j] : -1;
  }
  for (int i = 0; i <= cfg->n_r; ++i) T->r_edges[i] = cfg->r_edges[i];
  for (int i = 0; i <= cfg->n_p; ++i) T->p_edges[i] = cfg->p_edges[i];
  // logarithmic lookup over the float bit pattern of q: bucket = bits >> 17
  int base = 0;
  if (cfg->n_qbreak > 0) {
    unsigned bits;
    float lo = T->q_lo32[0] > 0.0f ? T->q_lo32[0] : 1e-30f;
    memcpy(&bits, &lo, 4);
    base = (int)(bits >> (23 - kLutMantBits)) - (1 << kLutMantBits);
    if (base < 0) base = 0;
  }
  *lut_base = base;
  const int n = cfg->n_qbreak;
  int n_dirty = 0;
  *short_tables = true;
  for (int b = 0; b < kLut; ++b) {
    unsigned lo_bits = (unsigned)(b + base) << (23 - kLutMantBits);
    unsigned hi_bits = (unsigned)(b + base + 1) << (23 - kLutMantBits);
    float lo, hi;
    memcpy(&lo, &lo_bits, 4);
    memcpy(&hi, &hi_bits, 4);
    if (!(lo < INFINITY)) {  // beyond the float range: walk (the short path never gets here)
      T->lut32[b] = 0x8000;
      T->lutw[b] = kLutReject;
      continue;
    }
    int iv = 0;
    while (iv < n && T->q_hi32[iv] <= lo) ++iv;
    bool clean = iv == n || T->q_lo32[iv] >= hi;
    // clean bucket: the bin itself (+1, 0 = not binned); otherwise the first
    // breakpoint to compare against, flagged
    T->lut32[b] = clean ? (unsigned short)(T->q_bin[iv] + 1) : (unsigned short)(iv | 0x8000);
    auto code = [&](int bin) { return bin >= 0 ? bin * cfg->n_p : kLutReject; };
    if (clean) {
      T->lutw[b] = (unsigned short)code(T->q_bin[iv]);
    } else {
      // the guard bands that meet this bucket, iv .. last, as one band
      int last = iv;
      while (last + 1 < n && T->q_lo32[last + 1] < hi) ++last;
      const float lo_band = T->q_lo32[iv], hi_band = T->q_hi32[last];
      const int below = code(T->q_bin[iv]), above = code(T->q_bin[last + 1]);
      int d = 0;
      while (d < n_dirty && !(T->qdirty[d].x == lo_band && T->qdirty[d].y == hi_band)) ++d;
      if (d == n_dirty) {
        if (n_dirty == MIA_MAX_BREAKS) {
          *short_tables = false;  // (too many: the generic path walks the breakpoints)
          d = 0;
        } else {
          float fb, fa;
          memcpy(&fb, &below, 4);
          memcpy(&fa, &above, 4);
          T->qdirty[n_dirty++] = make_float4(lo_band, hi_band, fb, fa);
        }
      }
      T->lutw[b] = (unsigned short)(d | 0x8000);
    }
  }
  // the short path's wrapped index: bucket 0 lies an octave below the first
  // guard band, so every q under the table has bin q_bin[0]
  T->lutw[kLut - 1] = (unsigned short)(n > 0 && T->q_bin[0] >= 0 ? T->q_bin[0] * cfg->n_p
                                                                   : (n > 0 ? kLutReject : T->lutw[kLut - 1]));
}

}  // namespace mia

using namespace mia;

extern "C" {

static int fail(mia_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}


int mia_version(void) { return 1; }

int mia_create(int device, mia_context** out) {
  if (!out) return MIA_ERR_ARG;
  *out = nullptr;
  mia_context* c = new mia_context();
  c->device = device;
  c->num_sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete c;
    return MIA_ERR_CUDA;
  }
  *out = c;
  return MIA_OK;
}

int mia_destroy(mia_context* ctx) {
  if (ctx) {
    free_profile_events(ctx);
    free_prep_streams(ctx);
  }
  delete ctx;
  return MIA_OK;
}

int mia_jackknife_cross_cov(mia_context* ctx, int n_real, int n_bins, const double* real_a, int64_t stride_a,
                            const double* real_b, int64_t stride_b, double* cov, double* std, void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (n_real < 1 || n_bins < 1 || n_bins > 4096 || !real_a || !real_b || !cov || !std || stride_a < n_bins ||
      stride_b < n_bins)
    return fail(ctx, MIA_ERR_ARG, "cross covariance: need n_real >= 1, 1 <= n_bins <= 4096, strides >= n_bins");
  const cudaError_t e = launch_cross_cov(n_real, n_bins, real_a, stride_a, real_b, stride_b, cov, std,
                                         static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(ctx, MIA_ERR_CUDA, std::string("cross covariance: ") + cudaGetErrorString(e));
  ctx->err.clear();
  return MIA_OK;
}

int mia_profile_pairs(mia_context* ctx, int n_slots) {
  if (!ctx || n_slots < 0) return MIA_ERR_ARG;
  free_profile_events(ctx);
  for (int i = 0; i < n_slots; ++i) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return fail(ctx, MIA_ERR_CUDA, "cudaEventCreate");
    if (cudaEventCreate(&b) != cudaSuccess) {
      cudaEventDestroy(a);
      return fail(ctx, MIA_ERR_CUDA, "cudaEventCreate");
    }
    ctx->prof_start.push_back(a);
    ctx->prof_stop.push_back(b);
  }
  return MIA_OK;
}

int mia_profile_read(mia_context* ctx, float* ms, int n, int* n_out) {
  if (!ctx || !ms || !n_out || n < 0) return MIA_ERR_ARG;
  const long long slots = (long long)ctx->prof_start.size();
  long long have = ctx->prof_count < slots ? ctx->prof_count : slots;
  if (have > n) have = n;
  for (long long k = 0; k < have; ++k) {  // oldest first among the last `have`
    const long long j = (ctx->prof_count - have + k) % slots;
    if (cudaEventSynchronize(ctx->prof_stop[j]) != cudaSuccess ||
        cudaEventElapsedTime(&ms[k], ctx->prof_start[j], ctx->prof_stop[j]) != cudaSuccess)
      return fail(ctx, MIA_ERR_CUDA, "pair-kernel timing events");
  }
  *n_out = (int)have;
  return MIA_OK;
}

const char* mia_last_error(const mia_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int mia_workspace_size(const mia_config* cfg, int64_t n_pos, int64_t n_shape, size_t* bytes) {
  if (!bytes) return MIA_ERR_ARG;
  return mia_batch_workspace_size(cfg, 1, &n_pos, &n_shape, bytes);
}

int mia_output_layout(const mia_config* cfg, mia_layout* lay) {
  if (!cfg || !lay) return MIA_ERR_ARG;
  if (cfg->n_r < 1 || cfg->n_r > MIA_MAX_BINS_R || cfg->n_p < 1 || cfg->n_p > MIA_MAX_BINS_P || cfg->l_subboxes < 0)
    return MIA_ERR_ARG;
  const int64_t nb = (int64_t)cfg->n_r * cfg->n_p, nr = cfg->n_r;
  const int64_t J = cfg->l_subboxes > 0 ? (int64_t)cfg->l_subboxes * cfg->l_subboxes * cfg->l_subboxes : 0;
  int64_t o = 0;
  auto take = [&](int64_t& f, int64_t n) {
    f = o;
    o += n;
  };
  take(lay->dd, (1 + J) * nb);
  take(lay->splus, (1 + J) * nb);
  take(lay->scross, nb);
  take(lay->variance, nb);
  take(lay->npos_jk, J);
  take(lay->nshape_jk, J);
  take(lay->R, 1);
  take(lay->R_jk, J);
  take(lay->rr, nb);
  take(lay->rr_jk, J * nb);
  take(lay->xi_gp, nb);
  take(lay->xi_gx, nb);
  take(lay->xi_gg, nb);
  take(lay->splusd, nb);
  take(lay->scrossd, nb);
  take(lay->sigmasq, nb);
  take(lay->xi_gp_jk, J * nb);
  take(lay->splusd_jk, J * nb);
  take(lay->xi_gg_jk, J * nb);
  take(lay->dd_jk, J * nb);
  take(lay->proj_gp, nr);
  take(lay->proj_gg, nr);
  take(lay->proj_gp_jk, J * nr);
  take(lay->proj_gg_jk, J * nr);
  take(lay->mean_gp, nr);
  take(lay->std_gp, nr);
  take(lay->cov_gp, nr * nr);
  take(lay->mean_gg, nr);
  take(lay->std_gg, nr);
  take(lay->cov_gg, nr * nr);
  take(lay->stats, 8);
  lay->total = o;
  return MIA_OK;
}

#define MIA_CUDA(call)                                                                             \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(ctx, MIA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

}  // extern "C"

namespace mia_batch {

// Workspace of a batch: a header (work counter, dataset descriptors, prefix of
// work-unit counts) followed by one dataset workspace per catalogue.
struct BatchPlan {
  std::vector<Plan> plans;
  std::vector<size_t> off;
  size_t ds_off = 0, prefix_off = 0, total = 0;
};

bool make_batch(const mia_config* cfg, int n, const mia_catalog* cats, BatchPlan* bp, std::string* why) {
  if (n < 1) {
    *why = "a batch needs at least one catalogue";
    return false;
  }
  bp->plans.resize(n);
  bp->off.resize(n);
  size_t o = align256(sizeof(BatchHeader));
  bp->ds_off = o;
  o = align256(o + sizeof(Dataset) * (size_t)n);
  bp->prefix_off = o;
  o = align256(o + sizeof(unsigned long long) * (size_t)(n + 1));
  for (int i = 0; i < n; ++i) {
    const mia_catalog* c = &cats[i];
    if (c->n_pos < 1 || c->n_shape < 1) {
      *why = "empty position or shape sample";
      return false;
    }
    if (!c->position || !c->weight || !c->position_shape || !c->axis_direction || !c->q || !c->weight_shape) {
      *why = "missing catalogue arrays";
      return false;
    }
    const char* w = "";
    if (!make_plan(cfg, c->n_pos, c->n_shape, &bp->plans[i], &w)) {
      *why = w;
      return false;
    }
    bp->off[i] = o;
    o = align256(o + bp->plans[i].total);
  }
  bp->total = o;
  return true;
}

size_t batch_bytes_for_sizes(const mia_config* cfg, int n, const int64_t* n_pos, const int64_t* n_shape, bool* ok) {
  size_t o = align256(sizeof(BatchHeader));
  o = align256(o + sizeof(Dataset) * (size_t)n);
  o = align256(o + sizeof(unsigned long long) * (size_t)(n + 1));
  *ok = true;
  for (int i = 0; i < n; ++i) {
    Plan p;
    const char* w = "";
    if (!make_plan(cfg, n_pos[i], n_shape[i], &p, &w)) {
      *ok = false;
      return 0;
    }
    o = align256(o + p.total);
  }
  return o;
}

void make_params(const mia_config* cfg, const Plan& plan, const Tables& T, int lut_base, Params* out) {
  Params& P = *out;
  memset(&P, 0, sizeof(P));
  P.kind = cfg->kind;
  P.membership = cfg->membership;
  P.precision = cfg->precision;
  P.los = cfg->los;
  P.ellipticity = cfg->ellipticity;
  P.want_variance = cfg->want_variance ? 1 : 0;
  P.n_r = cfg->n_r;
  P.n_p = cfg->n_p;
  P.nb = plan.nb;
  P.J = plan.J;
  P.n_sub = plan.n_sub;
  P.n_qbreak = cfg->n_qbreak;
  P.n_pbreak = cfg->n_pbreak;
  P.L = cfg->boxsize;
  P.halfL = cfg->boxsize / 2.0;
  P.Lf_hi = (float)cfg->boxsize;
  P.Lf_lo = (float)(cfg->boxsize - (double)P.Lf_hi);
  P.halfLf = (float)(cfg->boxsize / 2.0);
  P.rp_cut = cfg->rp_cut;
  P.rp_cut2 = cfg->rp_cut * cfg->rp_cut;
  for (int k = 0; k < 3; ++k) {
    P.axis[k] = plan.axis[k];
    P.n[k] = plan.n[k];
    P.R[k] = plan.R[k];
    P.full[k] = plan.full[k];
    P.s[k] = plan.s[k];
    P.inv_s[k] = (double)plan.n[k] / cfg->boxsize;
    P.m[k] = plan.m[k];
    P.nf[k] = plan.nf[k];
    P.Rf[k] = plan.Rf[k];
    P.sf[k] = plan.sf[k];
  }
  P.range_proj = plan.range_proj;
  P.range_los = plan.range_los;
  P.n_cells = plan.n_cells;
  P.shapes_per_unit = plan.shapes_per_unit;
  // the most jackknife regions (sub-boxes per dimension, multiplied) the fine
  // cells of a shape cell's neighbourhood can touch: work units per run
  P.reg_slots = 1;
  if (plan.J > 0) {
    for (int k = 0; k < 3; ++k) {
      const int cps = plan.nf[k] / plan.n_sub;
      const int span = plan.full[k] ? plan.nf[k] : plan.m[k] + 2 * plan.Rf[k];
      int m = (span + cps - 1) / cps + 1;
      if (m > plan.n_sub) m = plan.n_sub;
      P.reg_slots *= m;
    }
  }
  P.lut32_base = lut_base;
  const double p0 = cfg->p_edges[0], p1 = cfg->p_edges[cfg->n_p];
  P.p_lo32 = (float)p0;
  P.p_inv32 = (float)((double)cfg->n_p / (p1 - p0));
  {
    // guard band on t = (v - p_lo) * n_p / (p_hi - p_lo), in bins: four times a
    // bound on its FP32 error.  v = Pi carries the error of the hi/lo
    // difference; v = mu = Pi * rsqrt(r^2) adds rsqrtf (2 ulp) and r^2 (4.5e-7)
    const double u = 1.0 / 8388608.0;  // 2^-23
    const double inv = (double)cfg->n_p / (p1 - p0);
    const double vmax = cfg->kind == MIA_KIND_W ? plan.range_los : 1.0;
    double ev = cfg->kind == MIA_KIND_W ? vmax * u : vmax * 6e-7;
    double et = (ev + fabs(p0) * u * 0.5 + (vmax + fabs(p0)) * u * 0.5) * inv + cfg->n_p * u;
    P.p_guard = (float)fmin(0.25, fmax(4.0 * et, 1.0 / 1048576.0));
    P.p_half_in = 0.5f - P.p_guard;
    P.p_off32 = (float)(-p0 * inv);
    // short w path: t = z_s + off_p, with the shape's z_s = fma(z_hi, inv,
    // z_lo inv) and the position's off_p = fma(-z_lo, inv, fma(-z_hi, inv,
    // -p_lo inv)) in FP32.  Errors, in bins: the FP32 inverse width ((n_p +
    // 1) 2^-24 over the binned range), the rounding of -p_lo inv (|p_lo| inv
    // 2^-24), z_s's and off_p's FMA roundings (|z_s|, |off_p| <= (L + 2 reach
    // + |p_lo|) inv, 2^-24 of it each, three in all) and the rounding of t
    // ((n_p + 1) 2^-24); taken four times over
    const double lmax = (cfg->boxsize + 2.0 * plan.range_los + fabs(p0)) * inv;
    double ew = (2.0 * (cfg->n_p + 1) + 3.0 * lmax + fabs(p0) * inv) * (u * 0.5);
    // a line-of-sight reach that spans the box: t is brought to the minimum
    // image by adding or subtracting L n_p / (p_hi - p_lo) (its rounding and
    // that of the add); the wrap points -L/2 and L/2 are the Pi range's ends
    // or lie beyond them, so a pair near one is an edge or out of range
    const double L_t = cfg->boxsize * inv;
    P.short_wrap = cfg->kind == MIA_KIND_W && plan.full[2] && !plan.full[0] && !plan.full[1] &&
                   p0 >= -0.5 * cfg->boxsize && p1 <= 0.5 * cfg->boxsize;
    if (P.short_wrap) ew += 2.0 * L_t * (u * 0.5);
    P.t_wrap_lo = (float)((-0.5 * cfg->boxsize - p0) * inv);
    P.t_wrap_hi = (float)((0.5 * cfg->boxsize - p0) * inv);
    P.L_t = (float)L_t;
    P.p_guard_w = (float)fmin(0.25, fmax(4.0 * ew, 1.0 / 1048576.0));
  }
  P.c_guard = 1e-12f;
  P.wrap_guard = (float)(cfg->boxsize * 1e-5);
  const double pm = fmax(fabs(p0), fabs(p1));
  P.los_cut = cfg->kind == MIA_KIND_W ? f32_up(pm * (1.0 + 1e-5) + 1e-30) : INFINITY;
  P.zwin = f32_up(plan.range_los * (1.0 + 1e-5) + cfg->boxsize * 5e-7);
  P.range_los32 = f32_down(plan.range_los);
  const int nq = cfg->n_qbreak;
  P.q_cut = (nq > 0 && cfg->q_bin[nq] < 0) ? T.q_hi32[nq - 1] : INFINITY;
  // the short pair path looks up q <= q_cut only, in a bucket below the last one
  P.short_ok = 0;
  if (P.q_cut < INFINITY) {
    unsigned qb;
    memcpy(&qb, &P.q_cut, 4);
    P.short_ok = (qb >> (23 - kLutMantBits)) - (unsigned)lut_base < (unsigned)(kLut - 1) ? 1 : 0;
  }
  // each coordinate rounded to FP32 (2^-24 L), their difference and L - |d|
  // (2^-24 L each): 2^-22 L in all, taken four times over
  P.pre_margin = (float)(cfg->boxsize * (1.0 / 1048576.0));
  P.edge_capacity = plan.edge_capacity;
}

void make_dataset(const Plan& plan, void* base, const mia_catalog& cat, const mia_result& res, const mia_layout& lay,
                  Dataset* d) {
  bind_work(plan, base, &d->w);
  bind_arrays(plan, base, cat.n_pos, cat.n_shape, &d->w);
  d->w.edge_capacity = plan.edge_capacity;
  d->o.dd = res.out + lay.dd;
  d->o.splus = res.out + lay.splus;
  d->o.scross = res.out + lay.scross;
  d->o.variance = res.out + lay.variance;
  d->o.npairs = res.npairs;
}

__global__ void k_batch_status(const Dataset* ds, int n, BatchHeader* h) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  unsigned flags = 0;
  int first = -1;
  unsigned long long bad = ~0ULL;
  for (int i = 0; i < n; ++i) {
    const Status* st = ds[i].w.status;
    flags |= st->flags;
    if ((st->flags & kStatusRange) && first < 0) {
      first = i;
      bad = st->bad_index;
    }
  }
  h->flags = flags;
  h->first_bad = first;
  h->bad_index = bad;
}

}  // namespace mia_batch

using namespace mia_batch;

extern "C" {

int mia_batch_workspace_size(const mia_config* cfg, int n, const int64_t* n_pos, const int64_t* n_shape,
                             size_t* bytes) {
  if (!cfg || !n_pos || !n_shape || !bytes || n < 1) return MIA_ERR_ARG;
  bool ok = false;
  size_t b = batch_bytes_for_sizes(cfg, n, n_pos, n_shape, &ok);
  if (!ok) return MIA_ERR_ARG;
  *bytes = b;
  return MIA_OK;
}

int mia_batch_prepare(mia_context* ctx, const mia_config* cfg, int n, const mia_catalog* cats, void* workspace,
                      size_t workspace_bytes, const mia_result* results, void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (!cfg || !cats || !results) return fail(ctx, MIA_ERR_ARG, "null argument");
  BatchPlan bp;
  std::string why;
  if (!make_batch(cfg, n, cats, &bp, &why)) return fail(ctx, MIA_ERR_ARG, why);
  if (!workspace || workspace_bytes < bp.total || ((uintptr_t)workspace & 255))
    return fail(ctx, MIA_ERR_WORKSPACE, "workspace missing, not 256-byte aligned, or smaller than the size query");
  for (int i = 0; i < n; ++i)
    if (!results[i].out || !results[i].npairs) return fail(ctx, MIA_ERR_ARG, "null result buffer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MIA_CUDA(cudaSetDevice(ctx->device));
  if (n > 1) MIA_CUDA(make_prep_streams(ctx));
  mia_layout lay;
  mia_output_layout(cfg, &lay);
  unsigned char* b = static_cast<unsigned char*>(workspace);
  static thread_local Tables host_tables;
  static thread_local std::vector<Dataset> host_ds;
  int lut_base = 0;
  bool short_tables = true;
  build_tables(cfg, &host_tables, &lut_base, &short_tables);
  host_ds.resize(n);
  for (int i = 0; i < n; ++i) {
    make_dataset(bp.plans[i], b + bp.off[i], cats[i], results[i], lay, &host_ds[i]);
    MIA_CUDA(cudaMemcpyAsync(host_ds[i].w.tables, &host_tables, sizeof(Tables), cudaMemcpyHostToDevice, st));
  }
  MIA_CUDA(cudaMemcpyAsync(b + bp.ds_off, host_ds.data(), sizeof(Dataset) * (size_t)n, cudaMemcpyHostToDevice, st));
  MIA_CUDA(cudaStreamSynchronize(st));
  ctx->err.clear();
  return MIA_OK;
}

int mia_batch_enqueue(mia_context* ctx, const mia_config* cfg, int n, const mia_catalog* cats, void* workspace,
                      size_t workspace_bytes, const mia_result* results, void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (!cfg || !cats || !results) return fail(ctx, MIA_ERR_ARG, "null argument");
  BatchPlan bp;
  std::string why;
  if (!make_batch(cfg, n, cats, &bp, &why)) return fail(ctx, MIA_ERR_ARG, why);
  if (!workspace || workspace_bytes < bp.total || ((uintptr_t)workspace & 255))
    return fail(ctx, MIA_ERR_WORKSPACE, "workspace missing, not 256-byte aligned, or smaller than the size query");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  mia_layout lay;
  mia_output_layout(cfg, &lay);
  unsigned char* b = static_cast<unsigned char*>(workspace);
  int lut_base = 0;
  static thread_local Tables tq;  // host copy: only the guard values enter the launch parameters
  bool short_tables = true;
  build_tables(cfg, &tq, &lut_base, &short_tables);
  Params P;
  make_params(cfg, bp.plans[0], tq, lut_base, &P);
  if (!short_tables) P.short_ok = 0;
  BatchHeader* hdr = reinterpret_cast<BatchHeader*>(b);
  const Dataset* ds_dev = reinterpret_cast<const Dataset*>(b + bp.ds_off);
  unsigned long long* prefix = reinterpret_cast<unsigned long long*>(b + bp.prefix_off);
  MIA_CUDA(cudaMemsetAsync(hdr, 0, sizeof(BatchHeader), st));
  const size_t nb = (size_t)bp.plans[0].nb, J1 = (size_t)bp.plans[0].J + 1;
  {
  NvtxRange r("mia/prep");
  // catalogues of a batch prepare side by side on the context's streams
  // (forked from and joined back into `st`; mia_batch_prepare made them)
  const bool fan = n > 1 && ctx->prep_ready;
  if (fan) {
    MIA_CUDA(cudaEventRecord(ctx->fork, st));
    for (int k = 0; k < kPrepStreams; ++k) MIA_CUDA(cudaStreamWaitEvent(ctx->prep[k], ctx->fork, 0));
  }
  for (int i = 0; i < n; ++i) {
    const Plan& pl = bp.plans[i];
    unsigned char* base = b + bp.off[i];
    cudaStream_t sp = fan ? ctx->prep[i % kPrepStreams] : st;
    Dataset d;
    make_dataset(pl, base, cats[i], results[i], lay, &d);
    MIA_CUDA(cudaMemsetAsync(base + pl.off_status, 0, sizeof(Status), sp));
    MIA_CUDA(cudaMemsetAsync(&d.w.status->bad_index, 0xFF, sizeof(unsigned long long), sp));
    MIA_CUDA(cudaMemsetAsync(base + pl.off_pcount, 0, pl.off_tiles - pl.off_pcount, sp));
    MIA_CUDA(cudaMemsetAsync(base + pl.off_reg, 0, (size_t)(pl.J + 1) * 48 + 64, sp));
    MIA_CUDA(cudaMemsetAsync(base + pl.off_acc, 0, acc_bytes(pl), sp));
    MIA_CUDA(cudaMemsetAsync(results[i].out, 0, sizeof(double) * (size_t)lay.total, sp));
    MIA_CUDA(cudaMemsetAsync(results[i].npairs, 0, sizeof(unsigned long long) * J1 * nb, sp));
    MIA_CUDA(launch_prep(pl, P, cats[i], d.w, sp));
  }
  if (fan) {
    for (int k = 0; k < kPrepStreams; ++k) {
      MIA_CUDA(cudaEventRecord(ctx->join[k], ctx->prep[k]));
      MIA_CUDA(cudaStreamWaitEvent(st, ctx->join[k], 0));
    }
  }
  MIA_CUDA(launch_batch_prefix(ds_dev, n, P.reg_slots, prefix, st));
  }
  NvtxRange r_pairs("mia/pairs");
  const long long slot = ctx->prof_start.empty() ? -1 : ctx->prof_count % (long long)ctx->prof_start.size();
  if (slot >= 0) MIA_CUDA(cudaEventRecord(ctx->prof_start[slot], st));
  MIA_CUDA(launch_pairs(P, ds_dev, n, prefix, &hdr->wu_next, st, ctx->num_sms));
  if (slot >= 0) {
    MIA_CUDA(cudaEventRecord(ctx->prof_stop[slot], st));
    ++ctx->prof_count;
  }
  for (int i = 0; i < n; ++i) {
    Dataset d;
    make_dataset(bp.plans[i], b + bp.off[i], cats[i], results[i], lay, &d);
    if (P.precision == MIA_MIXED) {
      NvtxRange r("mia/edge_retest");
      MIA_CUDA(launch_edge_retest(P, d.w, d.o, st, ctx->num_sms));
    }
    NvtxRange r("mia/post");
    MIA_CUDA(launch_fixed_out(P, d.w, d.o, st));  // exact fixed-point sums -> the output doubles
    MIA_CUDA(launch_post(P, d.w, lay, results[i].out, cfg->volume, cats[i].n_pos, cats[i].n_shape, st));
  }
  ctx->err.clear();
  return MIA_OK;
}

int mia_batch_status(mia_context* ctx, int n, void* workspace, void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (!workspace || n < 1) return fail(ctx, MIA_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* b = static_cast<unsigned char*>(workspace);
  const Dataset* ds_dev = reinterpret_cast<const Dataset*>(b + align256(sizeof(BatchHeader)));
  BatchHeader* hdr = reinterpret_cast<BatchHeader*>(b);
  k_batch_status<<<1, 32, 0, st>>>(ds_dev, n, hdr);
  MIA_CUDA(cudaGetLastError());
  static thread_local BatchHeader hh;
  MIA_CUDA(cudaMemcpyAsync(&hh, hdr, sizeof(BatchHeader), cudaMemcpyDeviceToHost, st));
  MIA_CUDA(cudaStreamSynchronize(st));
  if (hh.flags & kStatusRange) {
    char buf[200];
    snprintf(buf, sizeof(buf),
             "coordinate outside [0, boxsize) or not finite (catalogue %d, first offending index %llu)",
             hh.first_bad, (unsigned long long)hh.bad_index);
    return fail(ctx, MIA_ERR_RANGE, buf);
  }
  if (hh.flags & kStatusOverflow)
    return fail(ctx, MIA_ERR_OVERFLOW, "edge re-test queue overflow; rerun in the FP64 form");
  ctx->err.clear();
  return MIA_OK;
}

int mia_measure_batch(mia_context* ctx, const mia_config* cfg, int n, const mia_catalog* cats, void* workspace,
                      size_t workspace_bytes, const mia_result* results, void* stream) {
  int rc = mia_batch_prepare(ctx, cfg, n, cats, workspace, workspace_bytes, results, stream);
  if (rc != MIA_OK) return rc;
  rc = mia_batch_enqueue(ctx, cfg, n, cats, workspace, workspace_bytes, results, stream);
  if (rc != MIA_OK) return rc;
  return mia_batch_status(ctx, n, workspace, stream);
}

int mia_measure(mia_context* ctx, const mia_config* cfg, const mia_catalog* cat, void* workspace,
                size_t workspace_bytes, const mia_result* res, void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (!cfg || !cat || !res || !res->out || !res->npairs) return fail(ctx, MIA_ERR_ARG, "null argument");
  return mia_measure_batch(ctx, cfg, 1, cat, workspace, workspace_bytes, res, stream);
}

// ---- entry point without device allocation ---------------------------------
//
// For callers that cannot allocate device memory (a host framework owning the
// whole GPU memory budget, or a loop where cudaMalloc's implicit device
// synchronisation is not allowed), mia_measure_static runs mia_measure on a
// scratch array compiled into this module.  In host code `g_static_scratch`
// is only a host-side handle: every call looks up its device address with
// cudaGetSymbolAddress, with the context's device current, and passes that on
// as the workspace (a device's first call also loads this module there; after
// a cudaDeviceReset the next call finds the array's new address).  Every call
// shares the array: mia_measure zeroes what must start at zero, and calls
// that overlap on the GPU race.

static __device__ __align__(256) unsigned char g_static_scratch[MIA_STATIC_SCRATCH_BYTES];

int mia_measure_static(mia_context* ctx, const mia_config* cfg, const mia_catalog* cat, const mia_result* res,
                       void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (!cfg || !cat || !res || !res->out || !res->npairs) return fail(ctx, MIA_ERR_ARG, "null argument");
  // the same checks and messages as mia_measure, then the size test
  BatchPlan bp;
  std::string why;
  if (!make_batch(cfg, 1, cat, &bp, &why)) return fail(ctx, MIA_ERR_ARG, why);
  if (bp.total > (size_t)MIA_STATIC_SCRATCH_BYTES) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "mia_measure_static: this measurement needs %zu bytes of scratch but the static scratch holds %llu; "
             "use mia_measure with a caller-provided workspace",
             bp.total, (unsigned long long)MIA_STATIC_SCRATCH_BYTES);
    return fail(ctx, MIA_ERR_WORKSPACE, buf);
  }
  void* base = nullptr;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaGetSymbolAddress(&base, g_static_scratch);
  if (e != cudaSuccess || !base)
    return fail(ctx, MIA_ERR_CUDA,
                std::string("mia_measure_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
  return mia_measure(ctx, cfg, cat, base, (size_t)MIA_STATIC_SCRATCH_BYTES, res, stream);
}

int mia_lc_workspace_size(const mia_lc_config* cfg, int64_t n_pos, int64_t n_shape, size_t* bytes) {
  LcPlan p;
  const char* why = nullptr;
  if (!bytes || !lc_plan(cfg, n_pos, n_shape, &p, &why)) return MIA_ERR_ARG;
  *bytes = p.total;
  return MIA_OK;
}

int mia_lc_count(mia_context* ctx, const mia_lc_config* cfg, const mia_lc_sample* pos, const mia_lc_sample* shp,
                 void* workspace, size_t workspace_bytes, double* out, int64_t* counts, uint32_t* status,
                 void* stream) {
  if (!ctx) return MIA_ERR_ARG;
  if (!cfg || !pos || !shp || !out || !counts || !status) return fail(ctx, MIA_ERR_ARG, "null argument");
  LcPlan p;
  const char* why = nullptr;
  if (!lc_plan(cfg, pos->n, shp->n, &p, &why)) return fail(ctx, MIA_ERR_ARG, std::string("lightcone: ") + why);
  if (pos->n > 0 && (!pos->ra || !pos->dec || !pos->chi || !pos->w || !pos->cos_dec))
    return fail(ctx, MIA_ERR_ARG, "lightcone: position arrays");
  if (shp->n > 0 && (!shp->ra || !shp->dec || !shp->chi || !shp->w)) return fail(ctx, MIA_ERR_ARG, "lightcone: shape arrays");
  if (shp->n > 0 && cfg->with_shapes && (!shp->e || !shp->c2a || !shp->s2a))
    return fail(ctx, MIA_ERR_ARG, "lightcone: shape terms (e, cos 2 phi, sin 2 phi)");
  if (cfg->n_patch > 0 && ((pos->n > 0 && !pos->patch) || (shp->n > 0 && !shp->patch)))
    return fail(ctx, MIA_ERR_ARG, "lightcone: patch labels");
  if (!workspace || workspace_bytes < p.total || ((uintptr_t)workspace & 255))
    return fail(ctx, MIA_ERR_WORKSPACE, "workspace missing, not 256-byte aligned, or smaller than the size query");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  MIA_CUDA(cudaSetDevice(ctx->device));
  MIA_CUDA(launch_lc(cfg, p, *pos, *shp, workspace, out, counts, status, ctx->num_sms, st));
  ctx->err.clear();
  return MIA_OK;
}

}  // extern "C"
