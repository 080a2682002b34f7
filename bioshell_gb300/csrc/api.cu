// api.cu -- the C ABI (include/bioshell_crmsd.h): contexts, device
// workspaces, host<->device staging, the call sequences of the plain and
// mixed paths (single set, batched sets, pair lists), the graph cache,
// metrics, and the host-side self-test hooks.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/syscall.h>
#include <unistd.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "crmsd_math.cuh"
#include "engine.h"

using namespace bs;

namespace bs {

bs_status set_err(bs_ctx *ctx, bs_status s, const char *fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return s;
}

bs_status cuda_err(bs_ctx *ctx, cudaError_t e, const char *what) {
  const bs_status s = (e == cudaErrorMemoryAllocation) ? BS_ERR_OOM : BS_ERR_CUDA;
  return set_err(ctx, s, "%s: %s", what, cudaGetErrorString(e));
}

bs_status ensure(bs_ctx *ctx, DevBuf &b, size_t bytes, const char *what) {
  if (bytes == 0) bytes = 16;
  if (b.cap >= bytes) return BS_OK;
  if (b.p) {
    cudaFree(b.p);
    ctx->used -= b.cap;
    b.p = nullptr;
    b.cap = 0;
  }
  ++ctx->gen;
  if (ctx->fail_alloc_after >= 0 && ctx->fail_alloc_after-- == 0)
    return set_err(ctx, BS_ERR_OOM, "%s: allocation of %zu bytes failed (injected by bs_debug_fail_alloc)", what, bytes);
  if (ctx->used + bytes > ctx->budget)
    return set_err(ctx, BS_ERR_BUDGET, "%s: %zu bytes would exceed the context budget (%zu of %zu in use)", what,
                   bytes, ctx->used, ctx->budget);
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return cuda_err(ctx, e, what);
  }
  ctx->used += bytes;
  b.cap = bytes;
  return BS_OK;
}

void release(bs_ctx *ctx, DevBuf &b) {
  if (b.p) {
    cudaFree(b.p);
    ctx->used -= b.cap;
    ++ctx->gen;
  }
  b.p = nullptr;
  b.cap = 0;
}

bool is_device_ptr(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

bool is_pinned_host(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

}  // namespace bs

namespace {

constexpr double kDefaultTol = 1e-4;                  // Angstrom, certified total |dRMSD| per pair
constexpr unsigned long long kFlagCap = 1ull << 24;  // queued exact recomputations
constexpr size_t kMaxGraphs = 16;
// banded read-back: results of at least 2^24 pairs, in about 16 bands
constexpr int64_t kBandMinPairs = 1ll << 24;
constexpr int kBands = 16;

#define CK(call, what)                                     \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return cuda_err(ctx, _e, what); \
  } while (0)

bs_status check_opts(bs_ctx *ctx, const bs_opts *o) {
  if (o->version != BS_OPTS_VERSION)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.version %u != %d", o->version, BS_OPTS_VERSION);
  if (o->precision != BS_PRECISION_PLAIN64 && o->precision != BS_PRECISION_MIXED)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.precision %d unknown", o->precision);
  if (o->layout != BS_LAYOUT_TRIANGLE && o->layout != BS_LAYOUT_SQUARE)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.layout %d unknown", o->layout);
  if (o->out_type != BS_OUT_F64 && o->out_type != BS_OUT_F32)
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.out_type %d unknown", o->out_type);
  if (o->flags & ~(BS_FLAG_NO_GRAPH | BS_FLAG_AUTOTUNE))
    return set_err(ctx, BS_ERR_INVALID_ARG, "bs_opts.flags %d unknown", o->flags);
  return BS_OK;
}

// Certified per-pair |dRMSD| budget: the kernels charge each pair its two
// structures' quantisation residuals (Minkowski) and give the fast path the
// rest (at least 1e-5 A).
float total_tolerance(const bs_opts &o) { return (float)(o.tolerance > 0 ? o.tolerance : kDefaultTol); }

size_t out_elems(int64_t n, int layout) {
  return layout == BS_LAYOUT_TRIANGLE ? (size_t)(n * (n - 1) / 2) : (size_t)n * (size_t)n;
}

float elapsed(bs_ctx *ctx, int a, int b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]) != cudaSuccess) {
    cudaGetLastError();
    return 0.f;
  }
  return ms;
}

bs_status ensure_stage(bs_ctx *ctx, size_t njobs) {
  const size_t bytes = std::max<size_t>(njobs, 1) * sizeof(Job);
  if (ctx->job_stage_cap >= bytes) return BS_OK;
  if (ctx->job_stage) cudaFreeHost(ctx->job_stage);
  if (ctx->job_back) cudaFreeHost(ctx->job_back);
  ctx->job_stage = ctx->job_back = nullptr;
  ctx->job_stage_cap = 0;
  ++ctx->gen;
  CK(cudaHostAlloc(&ctx->job_stage, bytes, cudaHostAllocDefault), "pinned job table");
  CK(cudaHostAlloc(&ctx->job_back, bytes, cudaHostAllocDefault), "pinned job table");
  ctx->job_stage_cap = bytes;
  return BS_OK;
}

void drop_graphs(bs_ctx *ctx) {
  for (auto &g : ctx->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  ctx->graphs.clear();
}

// Device workspaces for a plan; fills `b` (symmetric jobs: B side = A side).
bs_status prepare_buffers(bs_ctx *ctx, const Plan &plan, unsigned long long cap, MixedBuffers &b) {
  const int64_t ns = plan.nblocks * kBlockStructs, rows = plan.nblocks * kBlockRows;
  const int nj = (int)plan.jobs.size();
  bs_status s;
  if ((s = ensure(ctx, ctx->ctr, (size_t)ns * 3 * sizeof(long long), "centroids"))) return s;
  if ((s = ensure(ctx, ctx->info, (size_t)ns * sizeof(SInfo), "structure data"))) return s;
  for (int d = 0; d < 4; ++d)
    if ((s = ensure(ctx, ctx->dig[d], (size_t)rows * plan.pitch * sizeof(__nv_bfloat16), "digit matrices"))) return s;
  if ((s = ensure(ctx, ctx->jobs, (size_t)nj * sizeof(Job), "job table"))) return s;
  if ((s = ensure(ctx, ctx->jobmap, (size_t)plan.nblocks * sizeof(int), "block map"))) return s;
  if ((s = ensure(ctx, ctx->tiles, plan.tiles.size() * sizeof(Tile), "tile table"))) return s;
  if ((s = ensure(ctx, ctx->flags, (size_t)cap * sizeof(unsigned long long), "flag list"))) return s;
  if ((s = ensure_stage(ctx, nj))) return s;
  b = MixedBuffers{};
  b.ctr = static_cast<long long *>(ctx->ctr.p);
  b.info_a = static_cast<SInfo *>(ctx->info.p);
  b.info_b = b.info_a;
  for (int d = 0; d < 4; ++d) b.dig_a[d] = static_cast<__nv_bfloat16 *>(ctx->dig[d].p);
  for (int d = 0; d < 3; ++d) b.dig_b[d] = b.dig_a[d];
  b.pitch_a = b.pitch_b = plan.pitch;
  b.rows_a = b.rows_b = rows;
  b.jobs = static_cast<Job *>(ctx->jobs.p);
  b.jobmap = static_cast<int *>(ctx->jobmap.p);
  b.tiles = static_cast<Tile *>(ctx->tiles.p);
  b.flags = static_cast<unsigned long long *>(ctx->flags.p);
  b.flag_cap = cap;
  b.sc = static_cast<DevScalars *>(ctx->scal.p);
  b.wait_ns = ctx->wait_limit_ns;
  return BS_OK;
}

// Uploads the block map and tile table when they differ from the last call's.
bs_status upload_tables(bs_ctx *ctx, const Plan &plan, const MixedBuffers &b, const std::vector<int64_t> &key) {
  if (key == ctx->plan_key) return BS_OK;
  CK(cudaMemcpyAsync(b.jobmap, plan.jobmap.data(), plan.jobmap.size() * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream),
     "upload block map");
  if (!plan.tiles.empty())
    CK(cudaMemcpyAsync(b.tiles, plan.tiles.data(), plan.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice,
                       ctx->stream),
       "upload tile table");
  CK(cudaStreamSynchronize(ctx->stream), "upload tables");  // the vectors are pageable and short-lived
  ctx->plan_key = key;
  return BS_OK;
}

// The tile table of a symmetric plan depends only on each job's size, chain
// length, tile shape and row range, in call order.  A call whose jobs match
// the previous call's in these takes the context's table instead of
// rebuilding it (1.6 M tiles, ~3.6 ms of host time at 50,000 structures,
// during which the GPU would wait); the lease hands the table back to the
// context when the call ends.
struct TileLease {
  bs_ctx *ctx = nullptr;
  Plan *plan = nullptr;
  std::vector<int64_t> key;
  ~TileLease() {
    if (ctx && plan && !plan->tiles.empty()) {
      ctx->tile_cache.swap(plan->tiles);
      ctx->tile_key.swap(key);
    }
  }
};

std::string cached_symmetric_plan(bs_ctx *ctx, const std::vector<JobSpec> &specs, float tol, Plan &plan,
                                  TileLease &lease) {
  std::vector<int64_t> key;
  key.reserve(specs.size() * 5);
  for (const JobSpec &sp : specs) {
    key.push_back(sp.n);
    key.push_back(sp.L);
    key.push_back(sp.narrow);
    key.push_back(sp.row_lo);
    key.push_back(sp.row_hi);
  }
  const bool hit = !ctx->tile_cache.empty() && key == ctx->tile_key;
  const std::string m = make_symmetric_plan(specs, tol, !hit, plan);
  if (!m.empty()) return m;
  if (hit) {
    plan.tiles.swap(ctx->tile_cache);
    ctx->tile_key.clear();
  }
  lease.ctx = ctx;
  lease.plan = &plan;
  lease.key = std::move(key);
  return "";
}

std::vector<int64_t> plan_key(bs_ctx *ctx, const Plan &plan, unsigned long long cap) {
  // the wait bound is a kernel argument captured into the graph
  std::vector<int64_t> k = {(int64_t)ctx->gen, (int64_t)plan.jobs.size(), plan.nblocks, plan.pitch,
                            (int64_t)plan.tiles.size(), (int64_t)cap, (int64_t)ctx->wait_limit_ns};
  for (const Job &j : plan.jobs) {
    k.push_back(j.n);
    k.push_back(j.L);
    k.push_back(j.narrow);
  }
  return k;
}

// Runs the device sequence of a plan (graph replay when possible) and reads
// back the counters; the caller synchronises and calls finish_mixed.
bs_status launch_plan(bs_ctx *ctx, const Plan &plan, const MixedBuffers &b, bool use_graph,
                      const Readback *rb = nullptr) {
  const int nj = (int)plan.jobs.size();
  memcpy(ctx->job_stage, plan.jobs.data(), (size_t)nj * sizeof(Job));
  std::string m = get_encoder(&ctx->encode);
  if (!m.empty()) return set_err(ctx, BS_ERR_CUDA, "%s", m.c_str());
  CUtensorMap tm[7];
  m = encode_maps(ctx->encode, b, tm);
  if (!m.empty()) return set_err(ctx, BS_ERR_CUDA, "%s", m.c_str());
  const Job *stage = static_cast<const Job *>(ctx->job_stage);
  ctx->metrics.main_launches = plan.tiles.empty() ? 5 : rb ? 6 + 4 * (int)rb->tile_end.size() : 9;
  if (!use_graph || rb) {
    CK(enqueue_mixed(plan, b, stage, tm, ctx->num_sms, ctx->stream, &ctx->ev[1], false, nullptr, rb),
       "mixed-path launch");
    ctx->metrics.graph = 0;
  } else {
    const std::vector<int64_t> key = plan_key(ctx, plan, b.flag_cap);
    bs_ctx::Graph *hit = nullptr;
    for (auto &g : ctx->graphs)
      if (g.key == key) hit = &g;
    if (hit) {
      hit->last = ++ctx->tick;
      CK(cudaGraphLaunch(hit->exec, ctx->stream), "graph launch");
      ctx->metrics.graph = 2;
    } else {
      CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      const cudaError_t e = enqueue_mixed(plan, b, stage, tm, ctx->num_sms, ctx->stream, &ctx->ev[1], true);
      cudaGraph_t graph = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return cuda_err(ctx, e != cudaSuccess ? e : e2, "capture of the mixed-path sequence");
      }
      cudaGraphExec_t exec = nullptr;
      const cudaError_t e3 = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e3 != cudaSuccess) return cuda_err(ctx, e3, "graph instantiation");
      if (ctx->graphs.size() >= kMaxGraphs) {
        auto old = std::min_element(ctx->graphs.begin(), ctx->graphs.end(),
                                    [](const bs_ctx::Graph &x, const bs_ctx::Graph &y) { return x.last < y.last; });
        cudaGraphExecDestroy(old->exec);
        ctx->graphs.erase(old);
      }
      ctx->graphs.push_back(bs_ctx::Graph{key, exec, ++ctx->tick});
      CK(cudaGraphLaunch(exec, ctx->stream), "graph launch");
      ctx->metrics.graph = 1;
    }
  }
  CK(cudaMemcpyAsync(ctx->job_back, b.jobs, (size_t)nj * sizeof(Job), cudaMemcpyDeviceToHost, ctx->stream),
     "read job table");
  CK(cudaMemcpyAsync(ctx->sc_back, b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream), "read counters");
  return BS_OK;
}

// After synchronisation: errors and metrics of a mixed launch.
bs_status finish_mixed(bs_ctx *ctx, int nj) {
  const Job *jobs = static_cast<const Job *>(ctx->job_back);
  std::string msg;
  const bs_status s = collect_errors(*ctx->sc_back, jobs, nj, msg);
  if (s) return set_err(ctx, s, "%s", msg.c_str());
  float q = 0.f;
  for (int j = 0; j < nj; ++j) {
    float f;
    memcpy(&f, &jobs[j].qres_max_bits, 4);
    q = std::max(q, f);
  }
  ctx->metrics.pairs_refined = (int64_t)ctx->sc_back->flag_count;
  ctx->metrics.scale_exp = nj > 0 ? jobs[0].scale_exp : 0;
  ctx->metrics.quant_bound = 2.0 * q;  // worst pair's |dRMSD| from the grid
  ctx->metrics.jobs = nj;
  return BS_OK;
}

// ---------------------------------------------------------- autotuner
// Shape class of a structure set: 64-atom chain bucket and log2 of its size.
int64_t tune_key(int L, int64_t n) {
  int nb = 1;
  while ((1ll << nb) < n) ++nb;
  return (int64_t)(pitch_for(L) / kKChunk) * 64 + nb;
}

// Times 40 x 20 against 40 x 10 tiles on a synthetic set of the class (the
// class's upper size, at most 2048 structures, random 3.8 A chains of the
// set's length) and caches the faster; ties go to the wide tiles, which
// issue half the tensor-core instructions per pair.
bs_status tune_class(bs_ctx *ctx, int L, int64_t n_real, float tol, int &narrow, bool &tuned) {
  const int64_t key = tune_key(L, n_real);
  auto it = ctx->tune.find(key);
  tuned = false;
  if (it != ctx->tune.end()) {
    narrow = it->second;
    return BS_OK;
  }
  const int64_t n = std::max<int64_t>(2, std::min<int64_t>(1ll << (key % 64), 2048));
  std::vector<double> xyz((size_t)n * L * 3);
  uint64_t st = 0x9e3779b97f4a7c15ull ^ (uint64_t)key;
  auto rnd = [&]() {  // uniform in [-1, 1)
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (double)(st >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  };
  for (int64_t s = 0; s < n; ++s) {
    double p[3] = {0, 0, 0};
    for (int k = 0; k < L; ++k) {
      double d[3] = {rnd(), rnd(), rnd()};
      const double nd = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + 1e-9;
      for (int c = 0; c < 3; ++c) {
        p[c] += 3.8 * d[c] / nd;
        xyz[((size_t)s * L + k) * 3 + c] = p[c];
      }
    }
  }
  bs_status stt;
  if ((stt = ensure(ctx, ctx->pout, xyz.size() * 8, "autotuner coordinates"))) return stt;
  if ((stt = ensure(ctx, ctx->out, (size_t)(n * (n - 1) / 2) * 4, "autotuner result"))) return stt;
  CK(cudaMemcpy(ctx->pout.p, xyz.data(), xyz.size() * 8, cudaMemcpyHostToDevice), "autotuner coordinates");
  float best[2] = {1e30f, 1e30f};
  for (int v = 0; v < 2; ++v) {
    std::vector<JobSpec> specs{JobSpec{static_cast<const double *>(ctx->pout.p), n, L,
                                       OutDesc{ctx->out.p, n, n, kLayoutTriangle, 1}, v}};
    Plan plan;
    if (!make_symmetric_plan(specs, tol, true, plan).empty()) return set_err(ctx, BS_ERR_UNSUPPORTED, "autotuner plan");
    MixedBuffers b;
    if ((stt = prepare_buffers(ctx, plan, 4096, b))) return stt;
    ctx->plan_key.clear();
    if ((stt = upload_tables(ctx, plan, b, plan_key(ctx, plan, 4096)))) return stt;
    for (int rep = 0; rep < 3; ++rep) {
      if ((stt = launch_plan(ctx, plan, b, false))) return stt;
      CK(cudaStreamSynchronize(ctx->stream), "autotuner run");
      if ((stt = finish_mixed(ctx, 1))) return stt;
      if (rep > 0) best[v] = std::min(best[v], elapsed(ctx, 2, 3));
    }
  }
  ctx->plan_key.clear();
  narrow = best[1] < 0.97f * best[0] ? 1 : 0;
  ctx->tune[key] = narrow;
  tuned = true;
  return BS_OK;
}

// ---------------------------------------------------------- all-vs-all
struct SetIO {
  const double *xyz_dev;
  void *out_dev;
  size_t in_off, out_off;  // staging offsets (SIZE_MAX: caller's device memory)
  size_t in_bytes = 0;     // bytes of a host input to upload
};

bs_status plain_set(bs_ctx *ctx, const double *dxyz, int64_t n, int L, const OutDesc &od) {
  const int lp = lp_for(L);
  bs_status s;
  if ((s = ensure(ctx, ctx->ctrd, (size_t)n * 3 * sizeof(double), "centroids"))) return s;
  if ((s = ensure(ctx, ctx->y, (size_t)n * 3 * lp * sizeof(double), "centred coordinates"))) return s;
  if ((s = ensure(ctx, ctx->g, (size_t)n * sizeof(double), "norms"))) return s;
  DevScalars *sc = static_cast<DevScalars *>(ctx->scal.p);
  CK(launch_prep_plain(dxyz, n, L, lp, static_cast<double *>(ctx->ctrd.p), static_cast<double *>(ctx->y.p),
                       static_cast<double *>(ctx->g.p), &sc->err, ctx->stream),
     "prep plain");
  CK(launch_plain64_all(static_cast<const double *>(ctx->y.p), static_cast<const double *>(ctx->g.p), n, L, lp, od,
                        ctx->stream),
     "plain64 all-vs-all");
  return BS_OK;
}

// packed-triangle index of the first pair of row r (pairs (i, j), i < j)
inline int64_t row_off(int64_t n, int64_t r) { return r * n - r * (r + 1) / 2; }

// After a mixed launch: structure sets that no coordinate grid fits (the
// digit-1 products of chains beyond ~3,000 atoms exceed the exact range even
// in quarters of the chain; coordinates beyond +-32768 A) are computed on the
// plain FP64 path instead, into the same output, and their error is cleared.
// The mixed kernels wrote nothing of those sets.  A row-ranged call keeps
// the error: the plain path writes every row.
bs_status plain_fallback(bs_ctx *ctx, const std::vector<JobSpec> &specs, const std::vector<int> &set_of_spec,
                         const bs_set_desc *sets, const std::vector<SetIO> &io, const bs_opts &o, bool ranged) {
  Job *jobs = static_cast<Job *>(ctx->job_back);
  if (ctx->sc_back->err || ranged) return BS_OK;  // reported as they are
  const size_t esz = o.out_type == BS_OUT_F64 ? 8 : 4;
  bool any = false;
  for (size_t j = 0; j < specs.size(); ++j) {
    if ((jobs[j].err & kErrNonFinite) || !(jobs[j].err & kErrUnsupported)) continue;
    bs_status s = plain_set(ctx, specs[j].xyz, specs[j].n, specs[j].L, specs[j].out);
    if (s) return s;
    const int k = set_of_spec[j];
    if (io[k].out_off != SIZE_MAX)
      CK(cudaMemcpyAsync(sets[k].out, io[k].out_dev, out_elems(sets[k].n, o.layout) * esz, cudaMemcpyDeviceToHost,
                         ctx->stream),
         "copy result to host");
    jobs[j].err &= ~kErrUnsupported;
    ctx->metrics.pairs_plain += specs[j].n * (specs[j].n - 1) / 2;
    any = true;
  }
  if (any) CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  return BS_OK;
}

bs_status sets_impl(bs_ctx *ctx, const bs_set_desc *sets, int nsets, const bs_opts &o) {
  ctx->metrics = bs_metrics{};
  // a row range (bs_all_vs_all only; validated there): rows [rlo, rhi)
  const bool ranged = nsets == 1 && (o.row_begin != 0 || o.row_end != 0);
  const int64_t rlo = ranged ? o.row_begin : 0;
  const int64_t rhi = ranged ? (o.row_end > 0 ? std::min<int64_t>(o.row_end, sets[0].n) : sets[0].n) : 0;
  const size_t esz = o.out_type == BS_OUT_F64 ? 8 : 4;
  // tile shape per set (autotuner, mixed path), before anything is staged
  std::vector<int> narrow(nsets, 0);
  int tuned_classes = 0;
  if ((o.flags & BS_FLAG_AUTOTUNE) && o.precision == BS_PRECISION_MIXED) {
    for (int k = 0; k < nsets; ++k) {
      if (sets[k].n < 2) continue;
      bool tuned = false;
      const bs_status ts = tune_class(ctx, sets[k].L, sets[k].n, total_tolerance(o), narrow[k], tuned);
      if (ts) return ts;
      tuned_classes += tuned ? 1 : 0;
    }
    ctx->metrics = bs_metrics{};
  }
  // staging of host inputs / outputs
  std::vector<SetIO> io(nsets);
  size_t in_bytes = 0, out_bytes = 0;
  auto align = [](size_t v) { return (v + 255) & ~size_t(255); };
  int64_t pairs = 0;
  for (int k = 0; k < nsets; ++k) {
    const bs_set_desc &d = sets[k];
    io[k].in_off = io[k].out_off = SIZE_MAX;
    if (d.n < 2) continue;
    pairs += ranged ? row_off(d.n, rhi) - row_off(d.n, rlo) : d.n * (d.n - 1) / 2;
    if (!is_device_ptr(d.xyz)) {
      io[k].in_off = in_bytes;
      in_bytes = align(in_bytes + (size_t)d.n * d.L * 3 * sizeof(double));
    }
    if (!is_device_ptr(d.out)) {
      io[k].out_off = out_bytes;
      out_bytes = align(out_bytes + out_elems(d.n, o.layout) * esz);
    }
  }
  bs_status s;
  if (in_bytes && (s = ensure(ctx, ctx->xyz, in_bytes, "coordinates"))) return s;
  if (out_bytes && (s = ensure(ctx, ctx->out, out_bytes, "result buffer"))) return s;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  std::vector<JobSpec> specs;
  std::vector<int> set_of_spec;
  Readback rb;
  bool banded = false;
  for (int k = 0; k < nsets; ++k) {
    const bs_set_desc &d = sets[k];
    if (d.n < 2) continue;
    io[k].xyz_dev = d.xyz;
    if (io[k].in_off != SIZE_MAX) {
      double *dst = reinterpret_cast<double *>(static_cast<char *>(ctx->xyz.p) + io[k].in_off);
      const size_t bytes = (size_t)d.n * d.L * 3 * sizeof(double);
      ctx->metrics.bytes_h2d += (int64_t)bytes;
      io[k].xyz_dev = dst;
      io[k].in_bytes = bytes;  // copied below: up front, or band by band
    }
    io[k].out_dev = io[k].out_off != SIZE_MAX ? static_cast<char *>(ctx->out.p) + io[k].out_off : d.out;
    const int layout = o.layout == BS_LAYOUT_TRIANGLE ? kLayoutTriangle : kLayoutSquare;
    const OutDesc od{io[k].out_dev, d.n, d.n, layout, o.out_type};
    if (o.layout == BS_LAYOUT_SQUARE)
      CK(cudaMemset2DAsync(io[k].out_dev, (size_t)(d.n + 1) * esz, 0, esz, (size_t)d.n, ctx->stream), "zero diagonal");
    specs.push_back(JobSpec{io[k].xyz_dev, d.n, d.L, od, narrow[k]});
    if (ranged) {
      specs.back().row_lo = rlo;
      specs.back().row_hi = rhi;
    }
    set_of_spec.push_back(k);
    ctx->metrics.narrow_jobs += narrow[k];
  }
  // the uploads of host inputs, in set order, on the context's stream
  auto upload_all = [&]() -> bs_status {
    for (int k = 0; k < nsets; ++k)
      if (sets[k].n >= 2 && io[k].in_off != SIZE_MAX)
        CK(cudaMemcpyAsync(const_cast<double *>(io[k].xyz_dev), sets[k].xyz, io[k].in_bytes, cudaMemcpyHostToDevice,
                           ctx->stream),
           "copy coordinates to device");
    return BS_OK;
  };
  if (o.precision == BS_PRECISION_PLAIN64) {
    if ((s = upload_all())) return s;
    CK(cudaMemsetAsync(ctx->scal.p, 0, sizeof(DevScalars), ctx->stream), "clear counters");
    CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    for (const JobSpec &sp : specs)
      if ((s = plain_set(ctx, sp.xyz, sp.n, sp.L, sp.out))) return s;
    CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
    CK(cudaEventRecord(ctx->ev[4], ctx->stream), "event");
    CK(cudaMemcpyAsync(ctx->sc_back, ctx->scal.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream),
       "read counters");
    ctx->metrics.main_launches = 3 * (int)specs.size();
    ctx->metrics.jobs = (int)specs.size();
  } else if (!specs.empty()) {
    Plan plan;
    TileLease lease;
    const std::string m = cached_symmetric_plan(ctx, specs, total_tolerance(o), plan, lease);
    if (!m.empty()) return set_err(ctx, BS_ERR_UNSUPPORTED, "%s", m.c_str());
    if (ranged) {  // the overflow scan stays inside the range
      plan.scan_lo = row_off(specs[0].n, rlo);
      plan.scan_hi = row_off(specs[0].n, rhi);
    }
    unsigned long long cap = std::min<unsigned long long>(kFlagCap, std::max<int64_t>(pairs, 4096));
    if (o.flag_queue > 0) cap = std::min<unsigned long long>(cap, (unsigned long long)o.flag_queue);
    MixedBuffers b;
    if ((s = prepare_buffers(ctx, plan, cap, b))) return s;
    if ((s = upload_tables(ctx, plan, b, plan_key(ctx, plan, cap)))) return s;
    // one large triangle bound for pinned host memory: read back in row
    // bands while the later bands compute
    if (nsets == 1 && specs.size() == 1 && io[0].out_off != SIZE_MAX && o.layout == BS_LAYOUT_TRIANGLE &&
        pairs >= kBandMinPairs && is_pinned_host(sets[0].out) && !ranged) {
      if (!ctx->copy_stream) CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "copy stream");
      // the bands follow from the tile table and n: reused with the table
      std::vector<int64_t> bkey = lease.key;
      bkey.push_back(specs[0].n);
      bkey.push_back(kBands);
      if (bkey == ctx->band_key) {
        rb.tile_end = ctx->band_tile_end;
        rb.elem_end = ctx->band_elem_end;
      } else {
        make_bands(plan, specs[0].n, kBands, rb);
        ctx->band_key = std::move(bkey);
        ctx->band_tile_end = rb.tile_end;
        ctx->band_elem_end = rb.elem_end;
      }
      while (ctx->band_ev.size() < rb.tile_end.size() + 1) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "band event");
        ctx->band_ev.push_back(e);
      }
      rb.dev = static_cast<const char *>(io[0].out_dev);
      rb.host = static_cast<char *>(sets[0].out);
      rb.esz = esz;
      rb.copy = ctx->copy_stream;
      rb.ev = ctx->band_ev.data();
      banded = true;
    } else if (specs.size() > 1 && pairs >= kBandMinPairs) {
      // many sets with host outputs (all pinned): bands end on set
      // boundaries, and each band's sets are copied out while the later
      // bands compute
      bool pinned = false, pageable = false;
      for (int j = 0; j < (int)specs.size(); ++j) {
        const int k = set_of_spec[j];
        if (io[k].out_off == SIZE_MAX) continue;
        (is_pinned_host(sets[k].out) ? pinned : pageable) = true;
      }
      if (pinned && !pageable) {
        if (!ctx->copy_stream)
          CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "copy stream");
        make_set_bands(plan, kBands, rb);
        while (ctx->band_ev.size() < rb.tile_end.size() + 1) {
          cudaEvent_t e;
          CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "band event");
          ctx->band_ev.push_back(e);
        }
        int64_t t0 = 0;
        for (size_t band = 0; band < rb.tile_end.size(); ++band) {
          int last = -1;
          for (int64_t t = t0; t < rb.tile_end[band]; ++t) {
            const int j = plan.tiles[t].job;
            if (j == last) continue;
            last = j;
            const int k = set_of_spec[j];
            if (io[k].out_off == SIZE_MAX) continue;
            rb.copies[band].push_back(Readback::Copy{static_cast<const char *>(io[k].out_dev),
                                                     static_cast<char *>(sets[k].out),
                                                     out_elems(sets[k].n, o.layout) * esz});
          }
          t0 = rb.tile_end[band];
        }
        rb.copy = ctx->copy_stream;
        rb.ev = ctx->band_ev.data();
        banded = true;
        // inputs all in pinned host memory: each band's sets are uploaded on
        // a stream of their own and prepared when they land
        bool in_pinned = false, in_pageable = false;
        for (int j = 0; j < (int)specs.size(); ++j) {
          const int k = set_of_spec[j];
          if (io[k].in_off == SIZE_MAX) continue;
          (is_pinned_host(sets[k].xyz) ? in_pinned : in_pageable) = true;
        }
        if (in_pinned && !in_pageable) {
          if (!ctx->upload_stream)
            CK(cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking), "upload stream");
          while (ctx->up_ev.size() < rb.tile_end.size()) {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "upload event");
            ctx->up_ev.push_back(e);
          }
          rb.uploads.resize(rb.tile_end.size());
          int64_t u0 = 0;
          for (size_t band = 0; band < rb.tile_end.size(); ++band) {
            int last = -1;
            for (int64_t t = u0; t < rb.tile_end[band]; ++t) {
              const int j = plan.tiles[t].job;
              if (j == last) continue;
              last = j;
              const int k = set_of_spec[j];
              if (io[k].in_off != SIZE_MAX)
                rb.uploads[band].push_back(Readback::Upload{reinterpret_cast<char *>(const_cast<double *>(io[k].xyz_dev)),
                                                            reinterpret_cast<const char *>(sets[k].xyz),
                                                            io[k].in_bytes});
            }
            const Job &lj = plan.jobs[last];
            rb.struct_end.push_back(lj.first_a + blocks_for(lj.n) * kBlockStructs);
            u0 = rb.tile_end[band];
          }
          rb.struct_end.back() = plan.nblocks * kBlockStructs;
          rb.upload = ctx->upload_stream;
          rb.up_ev = ctx->up_ev.data();
        }
      }
    }
    if (rb.struct_end.empty() && (s = upload_all())) return s;
    s = launch_plan(ctx, plan, b, !(o.flags & BS_FLAG_NO_GRAPH), banded ? &rb : nullptr);
    if (s) {
      if (banded) cudaStreamSynchronize(ctx->copy_stream);
      if (ctx->upload_stream) cudaStreamSynchronize(ctx->upload_stream);
      return s;
    }
  } else {
    for (int k = 1; k <= 4; ++k) CK(cudaEventRecord(ctx->ev[k], ctx->stream), "event");
    memset(ctx->sc_back, 0, sizeof(DevScalars));
  }
  for (int k = 0; k < nsets; ++k) {
    const bs_set_desc &d = sets[k];
    if (d.n < 2 || io[k].out_off == SIZE_MAX) continue;
    size_t first = 0, bytes = out_elems(d.n, o.layout) * esz;
    if (ranged) {  // only the range's elements: the rest of the caller's buffer is left as it was
      first = (size_t)row_off(d.n, rlo) * esz;
      bytes = (size_t)(row_off(d.n, rhi) - row_off(d.n, rlo)) * esz;
    }
    if (!banded)
      CK(cudaMemcpyAsync(static_cast<char *>(d.out) + first, static_cast<const char *>(io[k].out_dev) + first, bytes,
                         cudaMemcpyDeviceToHost, ctx->stream),
         "copy result to host");
    ctx->metrics.bytes_d2h += (int64_t)bytes;
  }
  CK(cudaEventRecord(ctx->ev[5], ctx->stream), "event");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  if (o.precision == BS_PRECISION_PLAIN64) {
    if (ctx->sc_back->err & kErrNonFinite) return set_err(ctx, BS_ERR_NONFINITE, "input coordinates contain NaN or Inf");
  } else if (!specs.empty()) {
    if ((s = plain_fallback(ctx, specs, set_of_spec, sets, io, o, ranged))) return s;
    if ((s = finish_mixed(ctx, (int)specs.size()))) return s;
  }
  // single structures: their one square entry is the zero diagonal
  for (int k = 0; k < nsets; ++k) {
    const bs_set_desc &d = sets[k];
    if (d.n == 1 && o.layout == BS_LAYOUT_SQUARE) {
      const double z = 0.0;  // +0.0 has all-zero bits as f64 and as f32
      CK(cudaMemcpy(d.out, &z, esz, cudaMemcpyDefault), "write result");
    }
  }
  ctx->metrics.pairs = pairs;
  ctx->metrics.tuned_classes = tuned_classes;
  ctx->metrics.ms_h2d = elapsed(ctx, 0, 1);
  ctx->metrics.ms_prep = elapsed(ctx, 1, 2);
  ctx->metrics.ms_main = elapsed(ctx, 2, 3);
  ctx->metrics.ms_refine = elapsed(ctx, 3, 4);
  ctx->metrics.ms_d2h = elapsed(ctx, 4, 5);
  ctx->metrics.ms_total = elapsed(ctx, 0, 5);
  return BS_OK;
}

bs_status validate_sets(bs_ctx *ctx, const bs_set_desc *sets, int nsets) {
  for (int k = 0; k < nsets; ++k) {
    const bs_set_desc &d = sets[k];
    if (d.n < 0 || d.L < 1)
      return set_err(ctx, BS_ERR_INVALID_ARG, "set %d: n must be >= 0 and L >= 1 (n=%lld, L=%d)", k, (long long)d.n,
                     d.L);
    if (d.n > 0 && (!d.xyz || !d.out)) return set_err(ctx, BS_ERR_INVALID_ARG, "set %d: null coordinate or result pointer", k);
    if (d.n > (1LL << 31) - 1) return set_err(ctx, BS_ERR_UNSUPPORTED, "set %d: n above 2^31-1", k);
  }
  return BS_OK;
}

// ------------------------------------------------------------ pair list
bs_status pairs_impl(bs_ctx *ctx, const double *xyz, int64_t n, int L, const int64_t *ii, const int64_t *jj,
                     int64_t np, const bs_opts &o, double *out, float *levels_dbg) {
  ctx->metrics = bs_metrics{};
  const int lp = lp_for(L);
  bs_status s;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  const double *dxyz = xyz;
  if (!is_device_ptr(xyz)) {
    const size_t bytes = (size_t)n * (size_t)L * 3 * sizeof(double);
    if ((s = ensure(ctx, ctx->xyz, bytes, "coordinates"))) return s;
    CK(cudaMemcpyAsync(ctx->xyz.p, xyz, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy coordinates to device");
    ctx->metrics.bytes_h2d += (int64_t)bytes;
    dxyz = static_cast<const double *>(ctx->xyz.p);
  }
  const int64_t *dii = ii, *djj = jj;
  if (!is_device_ptr(ii)) {
    if ((s = ensure(ctx, ctx->pairs_i, (size_t)np * 8, "pair list"))) return s;
    CK(cudaMemcpyAsync(ctx->pairs_i.p, ii, (size_t)np * 8, cudaMemcpyHostToDevice, ctx->stream), "copy pair list");
    dii = static_cast<const int64_t *>(ctx->pairs_i.p);
  }
  if (!is_device_ptr(jj)) {
    if ((s = ensure(ctx, ctx->pairs_j, (size_t)np * 8, "pair list"))) return s;
    CK(cudaMemcpyAsync(ctx->pairs_j.p, jj, (size_t)np * 8, cudaMemcpyHostToDevice, ctx->stream), "copy pair list");
    djj = static_cast<const int64_t *>(ctx->pairs_j.p);
  }
  const bool out_dev = is_device_ptr(out);
  double *dout = out;
  if (!out_dev) {
    if ((s = ensure(ctx, ctx->pout, (size_t)np * 8, "pair results"))) return s;
    dout = static_cast<double *>(ctx->pout.p);
  }
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  if (o.precision == BS_PRECISION_PLAIN64) {
    if ((s = ensure(ctx, ctx->ctrd, (size_t)n * 3 * sizeof(double), "centroids"))) return s;
    if ((s = ensure(ctx, ctx->y, (size_t)n * 3 * lp * sizeof(double), "centred coordinates"))) return s;
    if ((s = ensure(ctx, ctx->g, (size_t)n * sizeof(double), "norms"))) return s;
    DevScalars *sc = static_cast<DevScalars *>(ctx->scal.p);
    CK(cudaMemsetAsync(sc, 0, sizeof(DevScalars), ctx->stream), "clear counters");
    CK(launch_prep_plain(dxyz, n, L, lp, static_cast<double *>(ctx->ctrd.p), static_cast<double *>(ctx->y.p),
                         static_cast<double *>(ctx->g.p), &sc->err, ctx->stream),
       "prep plain");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    CK(launch_plain64_pairs(static_cast<const double *>(ctx->y.p), static_cast<const double *>(ctx->g.p), n, L, lp,
                            dii, djj, np, dout, ctx->stream),
       "plain64 pairs");
    CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
    CK(cudaMemcpyAsync(ctx->sc_back, sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream), "read counters");
  } else {
    std::vector<JobSpec> specs{JobSpec{dxyz, n, L, OutDesc{dout, np, 0, kLayoutRect, 0}}};
    Plan plan;
    const std::string m = make_symmetric_plan(specs, total_tolerance(o), false, plan);
    if (!m.empty()) return set_err(ctx, BS_ERR_UNSUPPORTED, "%s", m.c_str());
    MixedBuffers b;
    if ((s = prepare_buffers(ctx, plan, 1024, b))) return s;
    ctx->plan_key.clear();
    if ((s = upload_tables(ctx, plan, b, plan_key(ctx, plan, 1024)))) return s;
    memcpy(ctx->job_stage, plan.jobs.data(), sizeof(Job));
    CUtensorMap tm[7];  // unused without tiles
    CK(enqueue_mixed(plan, b, static_cast<const Job *>(ctx->job_stage), tm, ctx->num_sms, ctx->stream, nullptr, false),
       "mixed preparation");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
    CK(launch_mixed_pairs(DigitsView{b.dig_a[0], b.dig_a[1], b.dig_a[2], b.pitch_a}, b.info_a, b.jobs, b.sc, dii, djj,
                          np, dout, levels_dbg, ctx->stream),
       "mixed pairs");
    CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
    CK(cudaMemcpyAsync(ctx->job_back, b.jobs, sizeof(Job), cudaMemcpyDeviceToHost, ctx->stream), "read job table");
    CK(cudaMemcpyAsync(ctx->sc_back, b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream), "read counters");
  }
  CK(cudaEventRecord(ctx->ev[4], ctx->stream), "event");
  if (!out_dev) {
    CK(cudaMemcpyAsync(out, dout, (size_t)np * 8, cudaMemcpyDeviceToHost, ctx->stream), "copy pair results");
    ctx->metrics.bytes_d2h += np * 8;
  }
  CK(cudaEventRecord(ctx->ev[5], ctx->stream), "event");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  if (o.precision == BS_PRECISION_PLAIN64) {
    if (ctx->sc_back->err & kErrNonFinite) return set_err(ctx, BS_ERR_NONFINITE, "input coordinates contain NaN or Inf");
  } else {
    if ((s = finish_mixed(ctx, 1))) return s;
  }
  ctx->metrics.pairs = np;
  ctx->metrics.ms_h2d = elapsed(ctx, 0, 1);
  ctx->metrics.ms_prep = elapsed(ctx, 1, 2);
  ctx->metrics.ms_main = elapsed(ctx, 2, 3);
  ctx->metrics.ms_d2h = elapsed(ctx, 4, 5);
  ctx->metrics.ms_total = elapsed(ctx, 0, 5);
  return BS_OK;
}

DevBuf *all_buffers(bs_ctx *ctx, std::vector<DevBuf *> &v) {
  v = {&ctx->xyz,     &ctx->out,    &ctx->ctr,   &ctx->info,  &ctx->dig[0], &ctx->dig[1], &ctx->dig[2],
       &ctx->dig[3],  &ctx->jobs,   &ctx->jobmap, &ctx->tiles, &ctx->flags,  &ctx->y,      &ctx->g,
       &ctx->ctrd,    &ctx->pairs_i, &ctx->pairs_j, &ctx->pout,
       &ctx->nbr_sink, &ctx->nbr_count, &ctx->nbr_ij, &ctx->nbr_d, &ctx->nbr_rows, &ctx->nbr_key, &ctx->nbr_tmp,
       &ctx->nbr_rowptr, &ctx->nbr_col, &ctx->nbr_dist, &ctx->hier_ws, &ctx->hier_tri, &ctx->hier_out,
       &ctx->sp_out};
  return nullptr;
}

// ------------------------------------------------------ neighbour lists
// The all-vs-all of one set in the neighbour layout: every pair with crmsd
// <= eps appended (both directions), then sorted into CSR rows on the
// device.  The append buffer starts at the previous call's size (or 2^22
// entries) and grows to the exact count once if it overflowed.
bs_status neighbors_impl(bs_ctx *ctx, const double *xyz, int64_t n, int L, float eps, const bs_opts &o,
                         int64_t *nnz_out) {
  ctx->metrics = bs_metrics{};
  ctx->nbr_n = -1;
  bs_status s;
  if ((s = ensure(ctx, ctx->nbr_rowptr, (size_t)(n + 1) * 8, "neighbour rows"))) return s;
  if (n < 2) {
    CK(cudaMemsetAsync(ctx->nbr_rowptr.p, 0, (size_t)(n + 1) * 8, ctx->stream), "clear rows");
    CK(cudaStreamSynchronize(ctx->stream), "synchronize");
    ctx->nbr_n = n;
    ctx->nbr_nnz = 0;
    *nnz_out = 0;
    return BS_OK;
  }
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  const double *dxyz = xyz;
  if (!is_device_ptr(xyz)) {
    const size_t bytes = (size_t)n * (size_t)L * 3 * sizeof(double);
    if ((s = ensure(ctx, ctx->xyz, bytes, "coordinates"))) return s;
    CK(cudaMemcpyAsync(ctx->xyz.p, xyz, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy coordinates to device");
    ctx->metrics.bytes_h2d += (int64_t)bytes;
    dxyz = static_cast<const double *>(ctx->xyz.p);
  }
  const unsigned long long all = (unsigned long long)n * (unsigned long long)(n - 1);
  unsigned long long cap = std::min(all, std::max(ctx->nbr_cap_hint, 1ull << 22));
  if ((s = ensure(ctx, ctx->nbr_sink, sizeof(NbrSink), "neighbour sink")) ||
      (s = ensure(ctx, ctx->nbr_count, 8, "neighbour count")))
    return s;
  unsigned long long count = 0;
  const int64_t pairs = n * (n - 1) / 2;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if ((s = ensure(ctx, ctx->nbr_ij, (size_t)cap * 8, "neighbour pairs")) ||
        (s = ensure(ctx, ctx->nbr_d, (size_t)cap * 4, "neighbour distances")))
      return s;
    const NbrSink sink{static_cast<unsigned long long *>(ctx->nbr_count.p), cap, static_cast<int2 *>(ctx->nbr_ij.p),
                       static_cast<float *>(ctx->nbr_d.p)};
    CK(cudaMemcpyAsync(ctx->nbr_sink.p, &sink, sizeof(sink), cudaMemcpyHostToDevice, ctx->stream), "sink");
    CK(cudaMemsetAsync(ctx->nbr_count.p, 0, 8, ctx->stream), "clear count");
    OutDesc od{ctx->nbr_sink.p, n, n, kLayoutNeighbors, 1};
    od.eps = eps;
    std::vector<JobSpec> specs{JobSpec{dxyz, n, L, od, 0}};
    Plan plan;
    TileLease lease;
    const std::string m = cached_symmetric_plan(ctx, specs, total_tolerance(o), plan, lease);
    if (!m.empty()) return set_err(ctx, BS_ERR_UNSUPPORTED, "%s", m.c_str());
    const unsigned long long fcap = std::min<unsigned long long>(kFlagCap, std::max<int64_t>(pairs, 4096));
    MixedBuffers b;
    if ((s = prepare_buffers(ctx, plan, fcap, b))) return s;
    if ((s = upload_tables(ctx, plan, b, plan_key(ctx, plan, fcap)))) return s;
    if ((s = launch_plan(ctx, plan, b, false))) return s;
    CK(cudaMemcpyAsync(&count, ctx->nbr_count.p, 8, cudaMemcpyDeviceToHost, ctx->stream), "read count");
    CK(cudaStreamSynchronize(ctx->stream), "synchronize");
    if ((s = finish_mixed(ctx, 1))) return s;
    if (ctx->sc_back->flag_count > fcap)
      return set_err(ctx, BS_ERR_UNSUPPORTED, "more than %llu pairs needed exact recomputation (neighbour lists)",
                     fcap);
    if (count <= cap) break;
    cap = count;
  }
  if (count > cap) return set_err(ctx, BS_ERR_INTERNAL, "neighbour count changed between attempts");
  ctx->nbr_cap_hint = count;
  if ((s = ensure(ctx, ctx->nbr_rows, (size_t)n * 16, "row counters")) ||
      (s = ensure(ctx, ctx->nbr_key, (size_t)count * 8, "neighbour keys")) ||
      (s = ensure(ctx, ctx->nbr_tmp, (size_t)count * 8, "neighbour keys")) ||
      (s = ensure(ctx, ctx->nbr_col, (size_t)count * 4, "neighbour columns")) ||
      (s = ensure(ctx, ctx->nbr_dist, (size_t)count * 4, "neighbour distances")))
    return s;
  CK(launch_neighbors_csr(static_cast<const int2 *>(ctx->nbr_ij.p), static_cast<const float *>(ctx->nbr_d.p),
                          (int64_t)count, n, ctx->num_sms, static_cast<int64_t *>(ctx->nbr_rowptr.p),
                          static_cast<int32_t *>(ctx->nbr_col.p), static_cast<float *>(ctx->nbr_dist.p),
                          static_cast<unsigned long long *>(ctx->nbr_rows.p),
                          static_cast<unsigned long long *>(ctx->nbr_key.p),
                          static_cast<unsigned long long *>(ctx->nbr_tmp.p), ctx->stream),
     "neighbour rows");
  CK(cudaEventRecord(ctx->ev[5], ctx->stream), "event");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  ctx->nbr_n = n;
  ctx->nbr_nnz = (int64_t)count;
  ctx->metrics.pairs = pairs;
  ctx->metrics.ms_prep = elapsed(ctx, 1, 2);
  ctx->metrics.ms_main = elapsed(ctx, 2, 3);
  ctx->metrics.ms_refine = elapsed(ctx, 3, 4);
  ctx->metrics.ms_total = elapsed(ctx, 0, 5);
  *nnz_out = (int64_t)count;
  return BS_OK;
}

}  // namespace

// ======================================================================
// C ABI
// ======================================================================
extern "C" {

BS_API int32_t bs_abi_version(void) { return BS_ABI_VERSION; }

BS_API const char *bs_status_string(bs_status s) {
  switch (s) {
    case BS_OK: return "ok";
    case BS_ERR_INVALID_ARG: return "invalid argument";
    case BS_ERR_CUDA: return "CUDA error";
    case BS_ERR_OOM: return "out of memory";
    case BS_ERR_TIMEOUT: return "device-side wait timed out";
    case BS_ERR_UNSUPPORTED: return "unsupported shape";
    case BS_ERR_NONFINITE: return "non-finite input";
    case BS_ERR_BUDGET: return "HBM budget exceeded";
    case BS_ERR_NO_DEVICE: return "no usable sm_103 GPU";
    case BS_ERR_INTERNAL: return "internal error";
    case BS_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
  }
}

BS_API const char *bs_last_error(const bs_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

BS_API void bs_opts_init(bs_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->version = BS_OPTS_VERSION;
  o->precision = BS_PRECISION_MIXED;
  o->layout = BS_LAYOUT_TRIANGLE;
  o->out_type = BS_OUT_F64;
  o->tolerance = 0.0;
  o->flags = 0;
}

BS_API bs_status bs_ctx_create(bs_ctx **out, int32_t device, size_t hbm_budget_bytes) {
  if (!out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return BS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return BS_ERR_INVALID_ARG;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BS_ERR_NO_DEVICE;
  if (!(prop.major == 10 && prop.minor == 3)) return BS_ERR_NO_DEVICE;  // built for sm_103a only
  bs_ctx *ctx = new (std::nothrow) bs_ctx();
  if (!ctx) return BS_ERR_OOM;
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return BS_ERR_CUDA;
  }
  if (mixed_tc_prepare() != cudaSuccess || prep_prepare() != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BS_ERR_CUDA;
  }
  for (auto &e : ctx->ev) cudaEventCreate(&e);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)(0.9 * (double)free_b);
  if (ensure(ctx, ctx->scal, sizeof(DevScalars), "scalars") != BS_OK ||
      cudaHostAlloc((void **)&ctx->sc_back, sizeof(DevScalars), cudaHostAllocDefault) != cudaSuccess) {
    bs_ctx_destroy(ctx);
    return BS_ERR_OOM;
  }
  *out = ctx;
  return BS_OK;
}

BS_API void bs_ctx_destroy(bs_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drop_graphs(ctx);
  std::vector<DevBuf *> bufs;
  all_buffers(ctx, bufs);
  bufs.push_back(&ctx->scal);
  for (DevBuf *b : bufs) release(ctx, *b);
  if (ctx->job_stage) cudaFreeHost(ctx->job_stage);
  if (ctx->job_back) cudaFreeHost(ctx->job_back);
  if (ctx->sc_back) cudaFreeHost(ctx->sc_back);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  for (cudaEvent_t e : ctx->band_ev) cudaEventDestroy(e);
  if (ctx->upload_stream) {
    cudaStreamSynchronize(ctx->upload_stream);
    cudaStreamDestroy(ctx->upload_stream);
  }
  for (cudaEvent_t e : ctx->up_ev) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

BS_API bs_status bs_ctx_trim(bs_ctx *ctx) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  drop_graphs(ctx);
  std::vector<DevBuf *> bufs;
  all_buffers(ctx, bufs);
  for (DevBuf *b : bufs) release(ctx, *b);
  ctx->plan_key.clear();
  std::vector<Tile>().swap(ctx->tile_cache);
  ctx->tile_key.clear();
  ctx->band_key.clear();
  return BS_OK;
}

BS_API void *bs_ctx_stream(const bs_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

BS_API bs_status bs_get_metrics(const bs_ctx *ctx, bs_metrics *out) {
  if (!ctx || !out) return BS_ERR_INVALID_ARG;
  *out = ctx->metrics;
  return BS_OK;
}

BS_API bs_status bs_all_vs_all(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const bs_opts *opts, void *out) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  bs_opts o;
  bs_opts_init(&o);
  if (opts) o = *opts;
  bs_status s = check_opts(ctx, &o);
  if (s) return s;
  bs_set_desc d{xyz, n, L, 0, out};
  if ((s = validate_sets(ctx, &d, 1))) return s;
  if (o.row_begin != 0 || o.row_end != 0) {
    const int64_t hi = o.row_end > 0 ? o.row_end : n;
    if (o.row_begin < 0 || o.row_begin % kBlockStructs || hi > n || o.row_begin > hi ||
        (hi % kBlockStructs && hi != n))
      return set_err(ctx, BS_ERR_INVALID_ARG,
                     "row range [%d, %d) of %lld structures: bounds must be multiples of 40 (the end may be n)",
                     o.row_begin, o.row_end, (long long)n);
    if (o.precision != BS_PRECISION_MIXED || o.layout != BS_LAYOUT_TRIANGLE)
      return set_err(ctx, BS_ERR_UNSUPPORTED, "row ranges need the mixed path and the packed triangle");
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return sets_impl(ctx, &d, 1, o);
}

BS_API bs_status bs_partition_rows(int64_t n, int32_t parts, int64_t *bounds) {
  if (n < 0 || parts < 1 || !bounds) return BS_ERR_INVALID_ARG;
  const int64_t total = n > 1 ? n * (n - 1) / 2 : 0;
  bounds[0] = 0;
  int64_t r = 0;
  for (int32_t p = 1; p < parts; ++p) {
    // the first block boundary at or past p / parts of the pairs
    const int64_t want = (int64_t)((double)total * p / parts);
    while (r < n && row_off(n, r) < want) r += kBlockStructs;
    bounds[p] = std::min(r, n);
  }
  bounds[parts] = n;
  return BS_OK;
}

BS_API bs_status bs_batched(bs_ctx *ctx, const bs_set_desc *sets, int32_t nsets, const bs_opts *opts) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (nsets < 0 || (nsets > 0 && !sets)) return set_err(ctx, BS_ERR_INVALID_ARG, "nsets < 0 or null set list");
  bs_opts o;
  bs_opts_init(&o);
  if (opts) o = *opts;
  bs_status s = check_opts(ctx, &o);
  if (s) return s;
  if ((s = validate_sets(ctx, sets, nsets))) return s;
  if (o.row_begin != 0 || o.row_end != 0) return set_err(ctx, BS_ERR_INVALID_ARG, "row ranges apply to bs_all_vs_all only");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return sets_impl(ctx, sets, nsets, o);
}

BS_API bs_status bs_neighbors(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, double eps, const bs_opts *opts,
                              int64_t *nnz) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (!nnz) return set_err(ctx, BS_ERR_INVALID_ARG, "null nnz");
  if (!(eps >= 0.0) || !(eps < 3.0e38)) return set_err(ctx, BS_ERR_INVALID_ARG, "eps must be finite and >= 0");
  bs_opts o;
  bs_opts_init(&o);
  if (opts) o = *opts;
  bs_status s = check_opts(ctx, &o);
  if (s) return s;
  if (o.precision != BS_PRECISION_MIXED)
    return set_err(ctx, BS_ERR_UNSUPPORTED, "neighbour lists are built by the mixed-precision path only");
  if (n < 0 || L < 1) return set_err(ctx, BS_ERR_INVALID_ARG, "n must be >= 0 and L >= 1");
  if (n > 0 && !xyz) return set_err(ctx, BS_ERR_INVALID_ARG, "null coordinates");
  if (n > (1LL << 31) - 1) return set_err(ctx, BS_ERR_UNSUPPORTED, "n above 2^31-1");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return neighbors_impl(ctx, xyz, n, L, (float)eps, o, nnz);
}

BS_API bs_status bs_hierarchical_gpu(bs_ctx *ctx, const void *tri, int64_t n, int32_t out_type, int32_t rule,
                                     int64_t *merges, float *merge_dist) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (n < 0 || (n > 1 && (!tri || !merges || !merge_dist))) return set_err(ctx, BS_ERR_INVALID_ARG, "bad argument");
  if (out_type != BS_OUT_F64 && out_type != BS_OUT_F32) return set_err(ctx, BS_ERR_INVALID_ARG, "out_type");
  if (rule < BS_LINK_SINGLE || rule > BS_LINK_WARD) return set_err(ctx, BS_ERR_INVALID_ARG, "unknown merge rule");
  if (n < 2) return BS_OK;
  if (n > (1LL << 20)) return set_err(ctx, BS_ERR_UNSUPPORTED, "n above 2^20");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  ctx->metrics = bs_metrics{};
  const int grid = hier_grid(ctx->num_sms);
  const size_t esz = out_type == BS_OUT_F64 ? 8 : 4;
  const size_t tri_bytes = (size_t)(n * (n - 1) / 2) * esz;
  bs_status s;
  if ((s = ensure(ctx, ctx->hier_ws, hier_workspace_bytes(n, grid), "clustering matrix")) ||
      (s = ensure(ctx, ctx->hier_out, (size_t)(n - 1) * 36, "clustering merges")))
    return s;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  const void *dtri = tri;
  if (!is_device_ptr(tri)) {
    if ((s = ensure(ctx, ctx->hier_tri, tri_bytes, "matrix staging"))) return s;
    CK(cudaMemcpyAsync(ctx->hier_tri.p, tri, tri_bytes, cudaMemcpyHostToDevice, ctx->stream), "copy matrix");
    dtri = ctx->hier_tri.p;
  }
  int64_t *dm = static_cast<int64_t *>(ctx->hier_out.p);
  float *dd = reinterpret_cast<float *>(dm + 4 * (n - 1));
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  int *derr = nullptr;
  CK(launch_hierarchical(dtri, out_type == BS_OUT_F64 ? 0 : 1, n, rule, ctx->hier_ws.p, grid, dm, dd, &derr,
                         ctx->wait_limit_ns, ctx->stream),
     "clustering launch");
  CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "read status");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  if (herr == 100) return set_err(ctx, BS_ERR_INTERNAL, "clustering: inconsistent merge pair");
  if (herr) return set_err(ctx, BS_ERR_TIMEOUT, "clustering: grid barrier of phase %d timed out", herr - 1);
  CK(cudaMemcpyAsync(merges, dm, (size_t)(n - 1) * 32, cudaMemcpyDefault, ctx->stream), "copy merges");
  CK(cudaMemcpyAsync(merge_dist, dd, (size_t)(n - 1) * 4, cudaMemcpyDefault, ctx->stream), "copy distances");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  ctx->metrics.ms_main = elapsed(ctx, 1, 2);
  ctx->metrics.ms_total = elapsed(ctx, 0, 2);
  return BS_OK;
}

BS_API bs_status bs_neighbors_get(bs_ctx *ctx, int64_t *row_ptr, int32_t *col, float *dist) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (ctx->nbr_n < 0) return set_err(ctx, BS_ERR_INVALID_ARG, "no neighbour lists: call bs_neighbors first");
  if (!row_ptr || (ctx->nbr_nnz > 0 && (!col || !dist))) return set_err(ctx, BS_ERR_INVALID_ARG, "null output");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  CK(cudaMemcpyAsync(row_ptr, ctx->nbr_rowptr.p, (size_t)(ctx->nbr_n + 1) * 8, cudaMemcpyDefault, ctx->stream),
     "copy rows");
  if (ctx->nbr_nnz > 0) {
    CK(cudaMemcpyAsync(col, ctx->nbr_col.p, (size_t)ctx->nbr_nnz * 4, cudaMemcpyDefault, ctx->stream), "copy columns");
    CK(cudaMemcpyAsync(dist, ctx->nbr_dist.p, (size_t)ctx->nbr_nnz * 4, cudaMemcpyDefault, ctx->stream),
       "copy distances");
  }
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  return BS_OK;
}

BS_API bs_status bs_tune_get(bs_ctx *ctx, int32_t L, int64_t n, int32_t *narrow) {
  if (!ctx || !narrow || L < 1 || n < 1) return BS_ERR_INVALID_ARG;
  auto it = ctx->tune.find(tune_key(L, n));
  *narrow = it == ctx->tune.end() ? -1 : it->second;
  return BS_OK;
}

BS_API bs_status bs_tune_set(bs_ctx *ctx, int32_t L, int64_t n, int32_t narrow) {
  if (!ctx || L < 1 || n < 1 || (narrow != 0 && narrow != 1)) return BS_ERR_INVALID_ARG;
  ctx->tune[tune_key(L, n)] = narrow;
  return BS_OK;
}

BS_API bs_status bs_tune_list(bs_ctx *ctx, int32_t *L_class, int64_t *n_class, int32_t *narrow, int32_t cap,
                              int32_t *count, int32_t *num_sms) {
  if (!ctx || !count || !num_sms || cap < 0 || (cap > 0 && (!L_class || !n_class || !narrow)))
    return BS_ERR_INVALID_ARG;
  *count = (int32_t)ctx->tune.size();
  *num_sms = ctx->num_sms;
  int32_t k = 0;
  for (const auto &kv : ctx->tune) {  // key = (pitch / 64) * 64 + ceil(log2 n)
    if (k >= cap) break;
    L_class[k] = (int32_t)(kv.first / 64) * kKChunk;
    n_class[k] = 1ll << (kv.first % 64);
    narrow[k] = kv.second;
    ++k;
  }
  return BS_OK;
}

BS_API bs_status bs_pairs(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii, const int64_t *jj,
                          int64_t npairs, const bs_opts *opts, double *out) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  bs_opts o;
  bs_opts_init(&o);
  if (opts) o = *opts;
  bs_status s = check_opts(ctx, &o);
  if (s) return s;
  if (n < 1 || L < 1 || npairs < 0) return set_err(ctx, BS_ERR_INVALID_ARG, "n >= 1, L >= 1, npairs >= 0 required");
  if (npairs == 0) return BS_OK;
  if (!xyz || !ii || !jj || !out) return set_err(ctx, BS_ERR_INVALID_ARG, "null pointer argument");
  if (!is_device_ptr(ii) && !is_device_ptr(jj)) {
    for (int64_t t = 0; t < npairs; ++t)
      if (ii[t] < 0 || ii[t] >= n || jj[t] < 0 || jj[t] >= n)
        return set_err(ctx, BS_ERR_INVALID_ARG, "pair %lld = (%lld, %lld) out of range [0, %lld)", (long long)t,
                       (long long)ii[t], (long long)jj[t], (long long)n);
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return pairs_impl(ctx, xyz, n, L, ii, jj, npairs, o, out, nullptr);
}

namespace {

// Superposition of a pair list (host or device pointers): staging as in
// pairs_impl, one warp per pair on the device.
bs_status superpose_impl(bs_ctx *ctx, const double *xyz, int64_t n, int L, const int64_t *ii, const int64_t *jj,
                         int64_t np, double *rot, double *trans, double *rmsd) {
  ctx->metrics = bs_metrics{};
  bs_status s;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  const double *dxyz = xyz;
  if (!is_device_ptr(xyz)) {
    const size_t bytes = (size_t)n * (size_t)L * 3 * sizeof(double);
    if ((s = ensure(ctx, ctx->xyz, bytes, "coordinates"))) return s;
    CK(cudaMemcpyAsync(ctx->xyz.p, xyz, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy coordinates to device");
    ctx->metrics.bytes_h2d += (int64_t)bytes;
    dxyz = static_cast<const double *>(ctx->xyz.p);
  }
  const int64_t *dii = ii, *djj = jj;
  if (!is_device_ptr(ii)) {
    if ((s = ensure(ctx, ctx->pairs_i, (size_t)np * 8, "pair list"))) return s;
    CK(cudaMemcpyAsync(ctx->pairs_i.p, ii, (size_t)np * 8, cudaMemcpyHostToDevice, ctx->stream), "copy pair list");
    dii = static_cast<const int64_t *>(ctx->pairs_i.p);
  }
  if (!is_device_ptr(jj)) {
    if ((s = ensure(ctx, ctx->pairs_j, (size_t)np * 8, "pair list"))) return s;
    CK(cudaMemcpyAsync(ctx->pairs_j.p, jj, (size_t)np * 8, cudaMemcpyHostToDevice, ctx->stream), "copy pair list");
    djj = static_cast<const int64_t *>(ctx->pairs_j.p);
  }
  // device outputs in place; host outputs staged (rot | trans | rmsd)
  const bool rot_dev = is_device_ptr(rot), trans_dev = is_device_ptr(trans), rmsd_dev = rmsd && is_device_ptr(rmsd);
  const size_t stage = (size_t)np * ((rot_dev ? 0 : 9) + (trans_dev ? 0 : 3) + (rmsd && !rmsd_dev ? 1 : 0));
  if (stage && (s = ensure(ctx, ctx->sp_out, stage * sizeof(double), "superposition results"))) return s;
  double *sp = static_cast<double *>(ctx->sp_out.p);
  double *drot = rot_dev ? rot : sp;
  double *dtrans = trans_dev ? trans : (rot_dev ? sp : sp + (size_t)np * 9);
  double *drmsd = !rmsd ? nullptr : rmsd_dev ? rmsd : sp + stage - (size_t)np;
  DevScalars *sc = static_cast<DevScalars *>(ctx->scal.p);
  CK(cudaMemsetAsync(sc, 0, sizeof(DevScalars), ctx->stream), "clear counters");
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
  CK(launch_superpose(dxyz, n, L, dii, djj, np, drot, dtrans, drmsd, &sc->err, ctx->num_sms, ctx->stream),
     "superposition");
  CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
  CK(cudaEventRecord(ctx->ev[4], ctx->stream), "event");
  if (!rot_dev) CK(cudaMemcpyAsync(rot, drot, (size_t)np * 72, cudaMemcpyDeviceToHost, ctx->stream), "copy rotations");
  if (!trans_dev)
    CK(cudaMemcpyAsync(trans, dtrans, (size_t)np * 24, cudaMemcpyDeviceToHost, ctx->stream), "copy translations");
  if (rmsd && !rmsd_dev)
    CK(cudaMemcpyAsync(rmsd, drmsd, (size_t)np * 8, cudaMemcpyDeviceToHost, ctx->stream), "copy rmsd");
  CK(cudaMemcpyAsync(ctx->sc_back, sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream), "read counters");
  CK(cudaEventRecord(ctx->ev[5], ctx->stream), "event");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  if (ctx->sc_back->err & kErrBounds) return set_err(ctx, BS_ERR_INVALID_ARG, "a pair index is out of range");
  if (ctx->sc_back->err & kErrNonFinite) return set_err(ctx, BS_ERR_NONFINITE, "input coordinates contain NaN or Inf");
  ctx->metrics.pairs = np;
  ctx->metrics.main_launches = 1;
  ctx->metrics.ms_h2d = elapsed(ctx, 0, 1);
  ctx->metrics.ms_main = elapsed(ctx, 2, 3);
  ctx->metrics.ms_d2h = elapsed(ctx, 4, 5);
  ctx->metrics.ms_total = elapsed(ctx, 0, 5);
  return BS_OK;
}

}  // namespace

BS_API bs_status bs_superpose_pairs(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii,
                                    const int64_t *jj, int64_t npairs, double *rot, double *trans, double *rmsd) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (n < 1 || L < 1 || npairs < 0) return set_err(ctx, BS_ERR_INVALID_ARG, "n >= 1, L >= 1, npairs >= 0 required");
  if (npairs == 0) return BS_OK;
  if (!xyz || !ii || !jj || !rot || !trans) return set_err(ctx, BS_ERR_INVALID_ARG, "null pointer argument");
  if (!is_device_ptr(ii) && !is_device_ptr(jj)) {
    for (int64_t t = 0; t < npairs; ++t)
      if (ii[t] < 0 || ii[t] >= n || jj[t] < 0 || jj[t] >= n)
        return set_err(ctx, BS_ERR_INVALID_ARG, "pair %lld = (%lld, %lld) out of range [0, %lld)", (long long)t,
                       (long long)ii[t], (long long)jj[t], (long long)n);
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  return superpose_impl(ctx, xyz, n, L, ii, jj, npairs, rot, trans, rmsd);
}

BS_API bs_status bs_superpose(bs_ctx *ctx, const double *a, const double *b, int32_t L, double *rot, double *trans,
                              double *rmsd) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (!a || !b || !rot || !trans || L < 1) return set_err(ctx, BS_ERR_INVALID_ARG, "null pointer or L < 1");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  const size_t one = (size_t)L * 3 * sizeof(double);
  bs_status s = ensure(ctx, ctx->xyz, 2 * one, "coordinates");
  if (s) return s;
  double *d = static_cast<double *>(ctx->xyz.p);
  CK(cudaMemcpyAsync(d, a, one, cudaMemcpyDefault, ctx->stream), "copy a");
  CK(cudaMemcpyAsync(d + (size_t)L * 3, b, one, cudaMemcpyDefault, ctx->stream), "copy b");
  const int64_t ii = 0, jj = 1;
  return superpose_impl(ctx, d, 2, L, &ii, &jj, 1, rot, trans, rmsd);
}

BS_API bs_status bs_crmsd(bs_ctx *ctx, const double *a, const double *b, int32_t L, double *out_rmsd) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (!a || !b || !out_rmsd || L < 1) return set_err(ctx, BS_ERR_INVALID_ARG, "null pointer or L < 1");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  const size_t one = (size_t)L * 3 * sizeof(double);
  bs_status s = ensure(ctx, ctx->xyz, 2 * one, "coordinates");
  if (s) return s;
  double *d = static_cast<double *>(ctx->xyz.p);
  CK(cudaMemcpyAsync(d, a, one, cudaMemcpyDefault, ctx->stream), "copy a");
  CK(cudaMemcpyAsync(d + (size_t)L * 3, b, one, cudaMemcpyDefault, ctx->stream), "copy b");
  const int64_t ii = 0, jj = 1;
  bs_opts o;
  bs_opts_init(&o);
  double r = 0.0;
  s = pairs_impl(ctx, d, 2, L, &ii, &jj, 1, o, &r, nullptr);
  if (s) return s;
  *out_rmsd = r;
  return BS_OK;
}

namespace {
// bs_host_alloc buffers placed with mmap + mbind (their sizes, for the free)
std::mutex g_near_mu;
std::map<void *, size_t> g_near;

// Page-locked memory on the host NUMA node of the current GPU: on systems
// where each CPU socket has its own GPU link (Grace), copies between a GPU
// and the other socket's memory cross the socket link and run at a fraction
// of the GPU link's rate.  cudaHostAlloc places the pages on the node of the
// calling thread, which may be the other socket.  The region is aligned to
// 2 MB and marked for transparent huge pages, so that where the kernel
// allows them the GPU's copies walk 2 MB pages instead of 4 KB ones.
// Returns null where the GPU reports no host NUMA node or the placement
// fails.
void *alloc_near_gpu(size_t bytes) {
#if defined(__linux__) && defined(SYS_mbind)
  int dev = 0, numa = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&numa, cudaDevAttrHostNumaId, dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  constexpr int kMaxNodes = 1024;
  constexpr int kBits = 8 * (int)sizeof(unsigned long);
  constexpr size_t kHuge = size_t(2) << 20;
  if (numa < 0 || numa >= kMaxNodes) return nullptr;
  const size_t span = (bytes + kHuge - 1) & ~(kHuge - 1);
  // reserve one huge page more, keep the 2 MB-aligned part
  char *raw = static_cast<char *>(mmap(nullptr, span + kHuge, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0));
  if (raw == MAP_FAILED) return nullptr;
  char *p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(raw) + kHuge - 1) & ~uintptr_t(kHuge - 1));
  if (p > raw) munmap(raw, (size_t)(p - raw));
  if (raw + span + kHuge > p + span) munmap(p + span, (size_t)(raw + span + kHuge - (p + span)));
#if defined(MADV_HUGEPAGE)
  madvise(p, span, MADV_HUGEPAGE);  // advice only: a kernel without THP ignores it
#endif
  unsigned long mask[kMaxNodes / kBits] = {};
  mask[numa / kBits] |= 1ul << (numa % kBits);
  const long kPreferred = 1;  // MPOL_PREFERRED: that node while it has free pages
  if (syscall(SYS_mbind, p, span, kPreferred, mask, (unsigned long)kMaxNodes + 1, 0ul) != 0 ||
      cudaHostRegister(p, span, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    munmap(p, span);
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_near_mu);
  g_near[p] = span;
  return p;
#else
  (void)bytes;
  return nullptr;
#endif
}
}  // namespace

BS_API bs_status bs_host_alloc(size_t bytes, void **out) {
  if (!out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  if (bytes == 0) return BS_OK;
  if ((*out = alloc_near_gpu(bytes)) != nullptr) return BS_OK;
  cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return e == cudaErrorMemoryAllocation ? BS_ERR_OOM : BS_ERR_CUDA;
  }
  return BS_OK;
}

BS_API bs_status bs_host_free(void *p) {
  if (!p) return BS_OK;
  size_t bytes = 0;
  {
    std::lock_guard<std::mutex> lk(g_near_mu);
    auto it = g_near.find(p);
    if (it != g_near.end()) {
      bytes = it->second;
      g_near.erase(it);
    }
  }
  if (bytes) {
    const bool ok = cudaHostUnregister(p) == cudaSuccess;
    munmap(p, bytes);
    return ok ? BS_OK : BS_ERR_CUDA;
  }
  return cudaFreeHost(p) == cudaSuccess ? BS_OK : BS_ERR_CUDA;
}

BS_API bs_status bs_debug_set_wait_limit(bs_ctx *ctx, int64_t ns) {
  if (!ctx || ns < 0) return BS_ERR_INVALID_ARG;
  ctx->wait_limit_ns = (uint64_t)ns;
  return BS_OK;
}

BS_API bs_status bs_debug_fail_alloc(bs_ctx *ctx, int64_t after) {
  if (!ctx || after < -1) return BS_ERR_INVALID_ARG;
  ctx->fail_alloc_after = after;
  return BS_OK;
}

BS_API bs_status bs_debug_tile_levels(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, float *levels) {
  if (!ctx || !xyz || !levels || n < 1 || L < 1) return BS_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  ctx->metrics = bs_metrics{};
  bs_status s;
  const size_t bytes = (size_t)n * (size_t)L * 3 * sizeof(double);
  if ((s = ensure(ctx, ctx->xyz, bytes, "coordinates"))) return s;
  CK(cudaMemcpyAsync(ctx->xyz.p, xyz, bytes, cudaMemcpyDefault, ctx->stream), "copy coordinates");
  const size_t nout = (size_t)n * (size_t)(n > 1 ? n - 1 : 1) / 2 + 1;
  if ((s = ensure(ctx, ctx->out, nout * 8, "result buffer"))) return s;
  std::vector<JobSpec> specs{
      JobSpec{static_cast<const double *>(ctx->xyz.p), n, L, OutDesc{ctx->out.p, n, n, kLayoutTriangle, 0}}};
  Plan plan;
  const std::string m = make_symmetric_plan(specs, (float)kDefaultTol, false, plan);
  if (!m.empty()) return set_err(ctx, BS_ERR_UNSUPPORTED, "%s", m.c_str());
  plan.tiles.push_back(Tile{0, 0, 0, 0});
  if (n > 20) plan.tiles.push_back(Tile{0, 1, 0, 0});
  MixedBuffers b;
  if ((s = prepare_buffers(ctx, plan, 4096, b))) return s;
  ctx->plan_key.clear();
  if ((s = upload_tables(ctx, plan, b, plan_key(ctx, plan, 4096)))) return s;
  ctx->plan_key.clear();
  if ((s = ensure(ctx, ctx->pout, (size_t)4 * 128 * 128 * sizeof(float), "level dump"))) return s;
  CK(cudaMemsetAsync(ctx->pout.p, 0, (size_t)4 * 128 * 128 * sizeof(float), ctx->stream), "clear level dump");
  memcpy(ctx->job_stage, plan.jobs.data(), sizeof(Job));
  std::string em = get_encoder(&ctx->encode);
  if (!em.empty()) return set_err(ctx, BS_ERR_CUDA, "%s", em.c_str());
  CUtensorMap tm[7];
  em = encode_maps(ctx->encode, b, tm);
  if (!em.empty()) return set_err(ctx, BS_ERR_CUDA, "%s", em.c_str());
  CK(enqueue_mixed(plan, b, static_cast<const Job *>(ctx->job_stage), tm, ctx->num_sms, ctx->stream, nullptr, false,
                   static_cast<float *>(ctx->pout.p)),
     "tensor-core tile");
  CK(cudaMemcpyAsync(levels, ctx->pout.p, (size_t)4 * 128 * 128 * sizeof(float), cudaMemcpyDefault, ctx->stream),
     "copy level dump");
  CK(cudaMemcpyAsync(ctx->job_back, b.jobs, sizeof(Job), cudaMemcpyDeviceToHost, ctx->stream), "read job table");
  CK(cudaMemcpyAsync(ctx->sc_back, b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream), "read counters");
  CK(cudaStreamSynchronize(ctx->stream), "synchronize");
  return finish_mixed(ctx, 1);
}

BS_API bs_status bs_debug_pair_levels(bs_ctx *ctx, const double *xyz, int64_t n, int32_t L, const int64_t *ii,
                                      const int64_t *jj, int64_t npairs, float *levels, double *rmsd) {
  if (!ctx || !xyz || !ii || !jj || !levels || !rmsd || n < 1 || L < 1 || npairs < 1) return BS_ERR_INVALID_ARG;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, BS_ERR_CUDA, "cudaSetDevice failed");
  for (int64_t t = 0; t < npairs; ++t)
    if (ii[t] < 0 || ii[t] >= n || jj[t] < 0 || jj[t] >= n) return set_err(ctx, BS_ERR_INVALID_ARG, "pair out of range");
  DevBuf lv;
  bs_status s = ensure(ctx, lv, (size_t)npairs * 36 * sizeof(float), "level dump");
  if (s) return s;
  bs_opts o;
  bs_opts_init(&o);
  s = pairs_impl(ctx, xyz, n, L, ii, jj, npairs, o, rmsd, static_cast<float *>(lv.p));
  if (s == BS_OK) {
    cudaError_t e = cudaMemcpy(levels, lv.p, (size_t)npairs * 36 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) s = cuda_err(ctx, e, "copy level dump");
  }
  release(ctx, lv);
  return s;
}

// ------------------------------------------------------------ test hooks
BS_API bs_status bs_selftest_bands(int64_t n, int32_t bands, int64_t *elem_end, int32_t cap, int32_t *count) {
  if (n < 2 || bands < 1 || !elem_end || !count || cap < 1) return BS_ERR_INVALID_ARG;
  std::vector<JobSpec> specs{JobSpec{nullptr, n, 16, OutDesc{nullptr, n, n, kLayoutTriangle, 0, 0.f, 0}}};
  Plan plan;
  if (!make_symmetric_plan(specs, (float)kDefaultTol, true, plan).empty()) return BS_ERR_UNSUPPORTED;
  Readback rb;
  make_bands(plan, n, bands, rb);
  *count = (int32_t)rb.elem_end.size();
  if (*count > cap) return BS_ERR_INVALID_ARG;
  for (int32_t i = 0; i < *count; ++i) elem_end[i] = rb.elem_end[i];
  return BS_OK;
}

BS_API bs_status bs_selftest_digits(const double *xyz, int32_t L, int32_t scale_exp, int32_t *digits,
                                    int64_t *g_exact, double *qres) {
  if (!xyz || !digits || !g_exact || !qres || L < 1) return BS_ERR_INVALID_ARG;
  double c[3] = {0, 0, 0};
  for (int k = 0; k < L; ++k)
    for (int d = 0; d < 3; ++d) c[d] += xyz[3 * k + d];
  for (int d = 0; d < 3; ++d) c[d] /= (double)L;
  long long g = 0;
  double res = 0.0;
  for (int k = 0; k < L; ++k)
    for (int d = 0; d < 3; ++d) {
      const double y = xyz[3 * k + d] - c[d];
      const double r = nearbyint(ldexp(y, -scale_exp));
      if (!(fabs(r) < 4194304.0)) return BS_ERR_UNSUPPORTED;
      const int q = (int)r;
      res += (y - ldexp(r, scale_exp)) * (y - ldexp(r, scale_exp));
      int a, b, e;
      bsm::split_digits(q, a, b, e);
      digits[(0 * 3 + d) * L + k] = a;
      digits[(1 * 3 + d) * L + k] = b;
      digits[(2 * 3 + d) * L + k] = e;
      g += (long long)q * q;
    }
  *g_exact = g;
  *qres = sqrt(res / (double)L);
  return BS_OK;
}

BS_API bs_status bs_selftest_epilogue(const float *levels, int64_t ga, int64_t gb, double qa, double qb, double d34,
                                      int32_t scale_exp, int32_t L, double tolerance, double *rmsd, int32_t *flag) {
  if (!levels || !rmsd || !flag || L < 1) return BS_ERR_INVALID_ARG;
  bsm::EpilogueIn in;
  for (int e = 0; e < 9; ++e) {
    in.s0[e] = levels[e];
    in.s1[e] = levels[9 + e];
    in.s2[e] = levels[18 + e];
    in.s3[e] = levels[27 + e];
  }
  in.ga = ga;
  in.gb = gb;
  in.gfa = (float)ga;
  in.gfb = (float)gb;
  in.qa = (float)qa;
  in.qb = (float)qb;
  int f = 0;
  const float r = bsm::pair_rmsd_fast(in, ldexpf(1.0f, 2 * scale_exp), (float)d34, L,
                                      (float)(tolerance > 0 ? tolerance : kDefaultTol), f);
  *rmsd = (double)r;
  *flag = f;
  return BS_OK;
}

BS_API bs_status bs_selftest_screen(const float *m9, double gsum, double de, double dr, int32_t scale_exp, int32_t L,
                                    float *lo, float *hi) {
  if (!m9 || !lo || !hi || L < 1) return BS_ERR_INVALID_ARG;
  bsm::screen_bracket(m9, (float)gsum, (float)de, (float)dr, ldexpf(1.0f, 2 * scale_exp), L, *lo, *hi);
  return BS_OK;
}

BS_API bs_status bs_selftest_exact(const int32_t *na, const int32_t *nb, int32_t L, int32_t scale_exp, double *rmsd) {
  if (!na || !nb || !rmsd || L < 1) return BS_ERR_INVALID_ARG;
  long long mh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  long long ga = 0, gb = 0;
  for (int k = 0; k < L; ++k)
    for (int x = 0; x < 3; ++x) {
      const long long ax = na[x * L + k];
      ga += ax * ax;
      const long long bx = nb[x * L + k];
      gb += bx * bx;
      for (int y = 0; y < 3; ++y) mh[3 * x + y] += ax * (long long)nb[y * L + k];
    }
  *rmsd = bsm::pair_rmsd_exact(mh, ga, gb, scale_exp, L);
  return BS_OK;
}

BS_API bs_status bs_selftest_superpose(const double *a, const double *b, int32_t L, double *rot, double *trans,
                                       double *rmsd) {
  if (!a || !b || !rot || !trans || L < 1) return BS_ERR_INVALID_ARG;
  double c[6] = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < L; ++k)
    for (int x = 0; x < 3; ++x) {
      c[x] += a[3 * k + x];
      c[3 + x] += b[3 * k + x];
    }
  for (int x = 0; x < 6; ++x) c[x] /= (double)L;
  double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < L; ++k)
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y) m[3 * x + y] += (a[3 * k + x] - c[x]) * (b[3 * k + y] - c[3 + y]);
  bsm::rotation_from_cov(m, rot);
  for (int x = 0; x < 3; ++x) trans[x] = c[x] - (rot[3 * x] * c[3] + rot[3 * x + 1] * c[4] + rot[3 * x + 2] * c[5]);
  if (rmsd) {
    double ss = 0.0;
    for (int k = 0; k < L; ++k)
      for (int x = 0; x < 3; ++x) {
        const double d = rot[3 * x] * b[3 * k] + rot[3 * x + 1] * b[3 * k + 1] + rot[3 * x + 2] * b[3 * k + 2] +
                         trans[x] - a[3 * k + x];
        ss += d * d;
      }
    *rmsd = sqrt(ss / (double)L);
  }
  return BS_OK;
}

}  // extern "C"
