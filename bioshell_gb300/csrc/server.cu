// server.cu -- the serving loop (include/bioshell_crmsd.h, bs_server_*).
//
// Library: one bucket per chain length, prepared once on the device with the
// mixed path's preparation (grid, digits, per-structure data) plus the plain
// path's FP64 centred coordinates; the bucket's grid and digit norms are the
// B side of every query job against it.
//
// Requests: a query is q structures of one bucket's length; its job is the
// rectangular block q x n_bucket on the tensor cores (query digits on the
// bucket's grid), written as a dense f32 block and reduced to the top_k
// nearest per query structure (topk.cu).  A clustering job is an all-vs-all
// of its own structures (f32 triangle) followed by OPTICS on a host worker.
//
// Scheduling (continuous batching): a scheduler thread polls the device
// slots (one CUDA stream each).  When a slot is free it takes the oldest
// queued request and, for a query, every other queued query of the same
// bucket up to max_batch_rows structures, and launches them as one batch
// (one preparation, one persistent tensor-core launch, one top-k launch).
// A batch is admitted only when its device memory fits the budget left by
// the other slots; batches in different slots run concurrently.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace bs {
namespace {

using Clock = std::chrono::steady_clock;
constexpr unsigned long long kServerFlagCap = 1ull << 20;
constexpr int kCandCap = 2048;  // screen candidates kept per query structure

// Growth of the calling thread's buffers during one batch (trace records).
thread_local int t_grow_dev = 0, t_grow_host = 0;
thread_local double t_grow_ms = 0.0;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
};

// The library index of a large bucket.  Every structure is joined to its
// nearest representative (exact crmsd at build time) and the bucket is
// stored in cluster order -- clusters contiguous, each sorted by distance
// to its representative -- so a library block of 20 holds one or two
// clusters.  The heads of the clusters (each representative and the members
// nearest to it) form a small set that a batch screens first: the k-th
// smallest upper bracket over the heads, T(q), bounds q's k-th nearest from
// above, and with d(x) an upper bound of crmsd(rep(x), x),
//   crmsd(q, x) >= crmsd(q, rep(x)) - d(x)     (triangle inequality),
// so a block whose members all have lo(q, rep) - d > T(q) + 2 tol holds
// none of q's top k, even after the certified per-pair error tol of the
// values that rank them.
struct Index {
  int nrep = 0;                // representatives (= clusters)
  int nhead = 0;               // head structures (every cluster's first members)
  DevBuf dig[4], info, tinfo;  // the heads' digit rows and data, on the bucket's grid
  int64_t rows = 0;            // digit rows of the head set
  DevBuf rep_slot;             // per cluster: its representative's slot in the head set (int32)
  DevBuf perm;                 // bucket position -> library index (int32)
  std::vector<int> c0, c1;     // per library block: first / last cluster (c0 -1: more than two)
  std::vector<float> d0, d1;   // per block: largest member bound d within c0 / c1
};

struct Bucket {
  int L = 0, lp = 0, pitch = 0;
  int64_t n = 0, rows = 0;
  int scale_exp = 0;
  float norm_b[3] = {0, 0, 0};
  float qres = 0.f;
  DevBuf dig[4], info;  // mixed path
  DevBuf tinfo;         // screen: truncated-structure data per structure
  DevBuf y, g;          // plain path: centred f64 [n][3][lp], squared norms
  bool indexed = false;
  Index ix;
};

// Library index of bucket position c (null: positions are library indices).
const int *bk_perm(const Bucket &bk) { return bk.indexed ? static_cast<const int *>(bk.ix.perm.p) : nullptr; }

struct Request {
  int64_t id = 0;
  int kind = 0;  // 0 query, 1 clustering job
  int bucket = -1;
  int L = 0;
  int64_t q = 0;
  std::vector<double> xyz;
  double eps = 0.0;
  int min_points = 0;
  std::vector<int64_t> idx;
  std::vector<double> val;
  std::vector<int64_t> labels;
  std::vector<float> tri;
  bs_status status = BS_OK;
  std::string err;
  bool done = false;
  Clock::time_point t_submit, t_done;
  int64_t pairs = 0;
  int64_t batch = -1;  // the batch that carried it (trace records)
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  cudaStream_t pst = nullptr;  // indexed screens: the pre-screen's high-priority stream
  cudaEvent_t pev = nullptr;
  // the slot's worker thread and its hand-off from the scheduler (server lock)
  std::thread worker;
  std::condition_variable cv;
  bool has_work = false, quit = false;
  bool busy = false;
  int kind = 0, bucket = -1;
  std::vector<Request *> reqs;
  std::vector<int64_t> row0;  // first dense row of each query job
  int64_t rows = 0;           // query structures in the batch
  int njobs = 0;
  bool screen = false;        // the batch ran the two-stage (screen + exact) top-k
  std::vector<int64_t> row_of;  // indexed screens: result row of query t of request j at row0[j] + t
  int64_t batch_id = -1;        // trace: sequence number of the batch in hand
  Clock::time_point t_hand;     // trace: when the scheduler handed it over
  // device
  DevBuf xyz, ctr, info, dig[4], jobs, jobmap, tiles, flags, scal, dense, topi, topv, y, g, ctrd;
  DevBuf tinfo, hist, thr, cand_j, cand_n, cand_v, rowtab, pre, prerep, segs;
  // pinned host
  HostBuf hxyz, htab, hjobs, hback, hsc, htopi, htopv, htri, hcand_n, hpre, hsegs;
  std::vector<void *> retired;  // replaced pinned buffers, freed when the server is destroyed
};

}  // namespace
}  // namespace bs

struct bs_server {
  int device = 0;
  int num_sms = 0;
  int top_k = 50;
  int max_inflight = 4;
  int64_t max_rows = 4096;
  int precision = BS_PRECISION_MIXED;
  float tol = 1e-4f;
  size_t budget = 0;
  std::atomic<size_t> used{0};  // in-flight device memory of the slots (workers grow their own buffers)
  std::vector<bs::Bucket> buckets;
  std::vector<std::unique_ptr<bs::Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_clus;
  std::deque<bs::Request *> queue, cluster_post;
  std::map<int64_t, bs::Request *> reqs;
  int64_t next_id = 1;
  bool stop = false;
  std::thread sched, clus;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  cudaMemPool_t pool = nullptr;  // the slots' device buffers
  std::string err;
  // stats
  std::vector<double> lat, clat;
  // optional trace (BS_SERVER_TRACE=<file>): one line per batch and request,
  // written when the server is destroyed
  std::string trace_path;
  std::vector<std::string> trace;
  int64_t qdone = 0, cdone = 0, pairs = 0, batches = 0, fallbacks = 0, rows_batched = 0;
  int64_t batch_seq = 0;  // trace: batch ids, never reset (the stats counter above is)
  std::atomic<int64_t> screened{0};  // updated by launches that run without the lock
  bs::Clock::time_point t0;
};

namespace bs {
namespace {

// ------------------------------------------------------------ memory
// Slot buffers come from the server's own stream-ordered pool: growing one
// frees and allocates on the slot's stream, so it never waits for the other
// slots' batches (cudaFree would synchronise the whole device).  The slot's
// stream is idle or nearly so when a buffer grows (its previous batch has
// completed on the host), and it is synchronised after the allocation so the
// buffer is usable from the slot's other stream too.
bool sv_ensure(bs_server *s, Slot &sl, DevBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.cap >= bytes) return true;
  const Clock::time_point t0 = Clock::now();
  if (b.p) {
    cudaFreeAsync(b.p, sl.st);
    s->used -= b.cap;
    b.p = nullptr;
    b.cap = 0;
  }
  bytes = bytes + bytes / 4;  // headroom: batches vary in size
  if (cudaMallocFromPoolAsync(&b.p, bytes, s->pool, sl.st) != cudaSuccess || cudaStreamSynchronize(sl.st) != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return false;
  }
  s->used += bytes;
  b.cap = bytes;
  ++t_grow_dev;
  t_grow_ms += ms_between(t0, Clock::now());
  return true;
}

void sv_release(bs_server *s, Slot &sl, DevBuf &b) {
  if (b.p) {
    cudaFreeAsync(b.p, sl.st);
    s->used -= b.cap;
  }
  b.p = nullptr;
  b.cap = 0;
}

// Pinned host buffers: a replaced buffer is kept until the server is
// destroyed (cudaFreeHost would synchronise the device).
bool host_ensure(Slot &sl, HostBuf &h, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (h.cap >= bytes) return true;
  const Clock::time_point t0 = Clock::now();
  if (h.p) sl.retired.push_back(h.p);
  h.p = nullptr;
  h.cap = 0;
  bytes = bytes + bytes / 4;
  if (cudaHostAlloc(&h.p, bytes, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  h.cap = bytes;
  ++t_grow_host;
  t_grow_ms += ms_between(t0, Clock::now());
  return true;
}

template <typename F>
void each_dev(Slot &sl, F f) {
  for (DevBuf *b : {&sl.xyz,   &sl.ctr,    &sl.info,   &sl.dig[0], &sl.dig[1], &sl.dig[2], &sl.dig[3],
                    &sl.jobs,  &sl.jobmap, &sl.tiles,  &sl.flags,  &sl.scal,   &sl.dense,  &sl.topi,
                    &sl.topv,  &sl.y,      &sl.g,      &sl.ctrd,   &sl.tinfo,  &sl.hist,   &sl.thr,
                    &sl.cand_j, &sl.cand_n, &sl.cand_v, &sl.rowtab, &sl.pre,   &sl.prerep, &sl.segs})
    f(*b);
}

template <typename F>
void each_host(Slot &sl, F f) {
  for (HostBuf *h : {&sl.hxyz, &sl.htab, &sl.hjobs, &sl.hback, &sl.hsc, &sl.htopi, &sl.htopv, &sl.htri,
                     &sl.hcand_n, &sl.hpre, &sl.hsegs})
    f(*h);
}

// Frees an idle slot's device buffers (its stream has nothing in flight)
// and gives the pool's unused memory back to the device.
void slot_release(bs_server *s, Slot &sl) {
  each_dev(sl, [&](DevBuf &b) { sv_release(s, sl, b); });
  cudaStreamSynchronize(sl.st);
  cudaMemPoolTrimTo(s->pool, 0);
}

size_t slot_bytes(Slot &sl) {
  size_t t = 0;
  each_dev(sl, [&](DevBuf &b) { t += b.cap; });
  return t;
}

// Device bytes a batch needs (without the headroom of sv_ensure).
size_t batch_bytes(const bs_server *s, const std::vector<Request *> &b) {
  if (b.empty()) return 0;
  const Request *r0 = b[0];
  const int L = r0->L;
  const int pitch = pitch_for(L), lp = lp_for(L);
  int64_t blocks = 0, rows = 0, tiles = 0;
  size_t xyz = 0;
  for (const Request *r : b) {
    blocks += blocks_for(r->q);
    rows += r->q;
    xyz += (size_t)r->q * L * 24;
  }
  size_t t = xyz + (size_t)blocks * kBlockStructs * (24 + 16 + 8) + (size_t)blocks * kBlockRows * pitch * 2 * 4 +
             b.size() * sizeof(Job) + (size_t)blocks * 4 + sizeof(DevScalars);
  if (r0->kind == 0) {
    const int64_t nb = s->buckets[r0->bucket].n;
    for (const Request *r : b) tiles += blocks_for(r->q) * ((nb + kBStructs - 1) / kBStructs);
    t += (size_t)tiles * sizeof(Tile) + kServerFlagCap * 8 + (size_t)rows * ((nb + 3) & ~int64_t(3)) * 4 +
         (size_t)rows * s->top_k * 12;
    if (s->precision == BS_PRECISION_PLAIN64) t += (size_t)rows * (3 * lp * 8 + 8 + 24);
    else t += (size_t)rows * (4 * kScreenBins + s->top_k * 12 + (size_t)kCandCap * 8 + 24);
  } else {
    const int64_t n = r0->q, nba = blocks_for(n), nbb = (n + kBStructs - 1) / kBStructs;
    for (int64_t i = 0; i < nba; ++i) tiles += std::max<int64_t>(0, nbb - 2 * i);
    t += (size_t)tiles * sizeof(Tile) + kServerFlagCap * 8 + (size_t)(n * (n - 1) / 2) * 4;
  }
  return t;
}

// ------------------------------------------------------------ library
bs_status build_bucket(bs_server *s, Bucket &bk, const double *xyz_in) {
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return BS_ERR_CUDA;
  bs_status status = BS_OK;
  DevBuf xyz, ctr, jobs, jobmap, scal, ctrd;
  auto fail = [&](bs_status e, const char *what) {
    status = e;
    s->err = what;
  };
  const size_t bytes = (size_t)bk.n * bk.L * 3 * sizeof(double);
  do {
    const double *dxyz = xyz_in;
    if (!is_device_ptr(xyz_in)) {
      if (cudaMalloc(&xyz.p, bytes) != cudaSuccess ||
          cudaMemcpyAsync(xyz.p, xyz_in, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        fail(BS_ERR_OOM, "library coordinates");
        break;
      }
      dxyz = static_cast<const double *>(xyz.p);
    }
    std::vector<JobSpec> specs{JobSpec{dxyz, bk.n, bk.L, OutDesc{nullptr, bk.n, bk.n, kLayoutTriangle, 1}}};
    Plan plan;
    const std::string m = make_symmetric_plan(specs, s->tol, false, plan);
    if (!m.empty()) {
      fail(BS_ERR_UNSUPPORTED, "library bucket shape unsupported");
      break;
    }
    plan.jobs[0].allow_long = 0;  // query tiles against the library use the normal layout
    bk.pitch = plan.pitch;
    bk.lp = lp_for(bk.L);
    bk.rows = plan.nblocks * kBlockRows;
    const int64_t ns = plan.nblocks * kBlockStructs;
    bool ok = cudaMalloc(&ctr.p, (size_t)ns * 24) == cudaSuccess && cudaMalloc(&bk.info.p, (size_t)ns * 16) == cudaSuccess &&
              cudaMalloc(&bk.tinfo.p, (size_t)ns * 8) == cudaSuccess &&
              cudaMalloc(&jobs.p, sizeof(Job)) == cudaSuccess && cudaMalloc(&jobmap.p, plan.nblocks * 4) == cudaSuccess &&
              cudaMalloc(&scal.p, sizeof(DevScalars)) == cudaSuccess;
    for (int d = 0; d < 4 && ok; ++d)
      ok = cudaMalloc(&bk.dig[d].p, (size_t)bk.rows * bk.pitch * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&bk.y.p, (size_t)bk.n * 3 * bk.lp * 8) == cudaSuccess &&
         cudaMalloc(&bk.g.p, (size_t)bk.n * 8) == cudaSuccess && cudaMalloc(&ctrd.p, (size_t)bk.n * 24) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      fail(BS_ERR_OOM, "library device memory");
      break;
    }
    MixedBuffers b{};
    b.ctr = static_cast<long long *>(ctr.p);
    b.info_a = static_cast<SInfo *>(bk.info.p);
    b.info_b = b.info_a;
    b.tinfo_a = static_cast<float2 *>(bk.tinfo.p);
    for (int d = 0; d < 4; ++d) b.dig_a[d] = static_cast<__nv_bfloat16 *>(bk.dig[d].p);
    for (int d = 0; d < 3; ++d) b.dig_b[d] = b.dig_a[d];
    b.pitch_a = b.pitch_b = bk.pitch;
    b.rows_a = b.rows_b = bk.rows;
    b.jobs = static_cast<Job *>(jobs.p);
    b.jobmap = static_cast<int *>(jobmap.p);
    b.sc = static_cast<DevScalars *>(scal.p);
    Job job = plan.jobs[0], back{};
    DevScalars sc{};
    CUtensorMap tm[7];  // no tiles: unused
    if (cudaMemcpyAsync(b.jobmap, plan.jobmap.data(), plan.jobmap.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        enqueue_mixed(plan, b, &job, tm, s->num_sms, st, nullptr, false) != cudaSuccess ||
        launch_prep_plain(dxyz, bk.n, bk.L, bk.lp, static_cast<double *>(ctrd.p), static_cast<double *>(bk.y.p),
                          static_cast<double *>(bk.g.p), &b.sc->err, st) != cudaSuccess ||
        cudaMemcpyAsync(&back, b.jobs, sizeof(Job), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&sc, b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      fail(BS_ERR_CUDA, "library preparation");
      break;
    }
    std::string msg;
    const bs_status e = collect_errors(sc, &back, 1, msg);
    if (e) {
      status = e;
      s->err = "library: " + msg;
      break;
    }
    bk.scale_exp = back.scale_exp;
    const int pick = back.scale_exp - back.scale_base;
    for (int d = 0; d < 3; ++d) bk.norm_b[d] = (float)(sqrt((double)back.norm[pick][d]) * (1.0 + 1e-6));
    memcpy(&bk.qres, &back.qres_max_bits, 4);
  } while (false);
  for (DevBuf *d : {&xyz, &ctr, &jobs, &jobmap, &scal, &ctrd})
    if (d->p) cudaFree(d->p);
  cudaStreamDestroy(st);
  return status;
}

// ------------------------------------------------------------ batches
// Half-precision bits -> float (the packed screen brackets).
float half_bits_to_float(uint32_t h) {
  const uint32_t sgn = (h >> 15) & 1u, e = (h >> 10) & 31u, m = h & 1023u;
  float v;
  if (e == 0) v = ldexpf((float)m, -24);
  else if (e == 31) v = m ? NAN : INFINITY;
  else v = ldexpf((float)(m | 1024u), (int)e - 25);
  return sgn ? -v : v;
}

// Tiles of one query batch: query blocks x library column blocks, column
// block by column block (strips for chains the strip kernel takes).  need
// (optional) lists the library blocks each query block has to see.
void batch_tiles(const bs_server *s, const Plan &plan_in, int64_t blk, int64_t nbb, int nk16, bool strips,
                 const std::vector<std::vector<int64_t>> *need, std::vector<Tile> &tiles) {
  tiles.clear();
  if (strips) {
    const int64_t total = blk * nbb;
    const int64_t run =
        std::max<int64_t>(8, std::min<int64_t>(4096, (total + 12 * s->num_sms - 1) / (12 * s->num_sms)));
    if (!need) {
      for (int64_t J = 0; J < nbb; J += run)
        for (int64_t I = 0; I < blk; ++I) {
          const int64_t cnt = std::min(run, nbb - J);
          tiles.push_back(Tile{(int)I, (int)J, plan_in.jobmap[I], nk16 | (int)(cnt << 16)});
        }
      return;
    }
    // runs of consecutive needed blocks, at most `run` long
    const int64_t prun = std::max<int64_t>(8, std::min<int64_t>(run, 64));
    for (int64_t I = 0; I < blk; ++I) {
      const std::vector<int64_t> &v = (*need)[I];
      for (size_t a = 0; a < v.size();) {
        size_t e = a + 1;
        while (e < v.size() && v[e] == v[e - 1] + 1 && (int64_t)(e - a) < prun) ++e;
        tiles.push_back(Tile{(int)I, (int)v[a], plan_in.jobmap[I], nk16 | (int)((int64_t)(e - a) << 16)});
        a = e;
      }
    }
    return;
  }
  if (!need) {
    tiles.reserve((size_t)(blk * nbb));
    for (int64_t J = 0; J < nbb; ++J)
      for (int64_t I = 0; I < blk; ++I) tiles.push_back(Tile{(int)I, (int)J, plan_in.jobmap[I], 0});
    return;
  }
  for (int64_t I = 0; I < blk; ++I)
    for (int64_t J : (*need)[I]) tiles.push_back(Tile{(int)I, (int)J, plan_in.jobmap[I], 0});
}

// Per row r of a [rows][ld] block of packed brackets: the words at the
// representatives' slots, into out[r][c].
__global__ void k_gather_cols(const uint32_t *__restrict__ pre, int64_t ld, const int *__restrict__ slot, int R,
                              int64_t rows, uint32_t *__restrict__ out) {
  const int64_t r = blockIdx.y;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < R; c += gridDim.x * blockDim.x)
    out[r * R + c] = pre[r * ld + slot[c]];
}

// Indexed screens, phase 1: the batch's queries (request order) against the
// bucket's head set on the tensor cores; the k-th smallest upper bracket of
// each row (the screen selection's threshold) and the brackets against the
// representatives are read back.  On the host each request's queries are
// ordered by nearest representative (so a query block holds similar
// queries) and each query block gets the library blocks it cannot rule out.
// Returns false when the index cannot be used for this batch (a job reported
// an error): the batch then runs unpruned.
bool index_prescreen(bs_server *s, Slot &sl, const Plan &base, int64_t blk, int64_t rows, const double *dx,
                     const std::vector<size_t> &xoff, std::vector<std::vector<int>> &order,
                     std::vector<std::vector<int64_t>> &need) {
  const Bucket &bk = s->buckets[sl.bucket];
  const Index &ix = bk.ix;
  const int nj = (int)base.jobs.size(), R = ix.nrep, H = ix.nhead, nk16 = bk.lp / 16, k = s->top_k;
  const int64_t ldh = (H + 3) & ~3, nbh = (H + kBStructs - 1) / kBStructs;
  Plan p1 = base;
  p1.strips = nk16 <= screen_strip_max_nk16();
  batch_tiles(s, p1, blk, nbh, nk16, p1.strips, nullptr, p1.tiles);
  if (!sv_ensure(s, sl, sl.pre, (size_t)rows * ldh * 4) || !sv_ensure(s, sl, sl.prerep, (size_t)rows * (R + 1) * 4) ||
      !host_ensure(sl, sl.hpre, (size_t)rows * (R + 1) * 4) || !sv_ensure(s, sl, sl.tiles, p1.tiles.size() * sizeof(Tile)) ||
      !host_ensure(sl, sl.htab, p1.jobmap.size() * 4 + p1.tiles.size() * sizeof(Tile)))
    return false;
  uint32_t *pre = static_cast<uint32_t *>(sl.pre.p);
  for (int j = 0; j < nj; ++j) {
    p1.jobs[j].xyz = dx + xoff[j];
    p1.jobs[j].n_b = H;
    p1.jobs[j].out = OutDesc{pre + sl.row0[j] * ldh, p1.jobs[j].n, ldh, kLayoutRect, 1};
  }
  memcpy(sl.hjobs.p, p1.jobs.data(), (size_t)nj * sizeof(Job));
  char *ht = static_cast<char *>(sl.htab.p);
  memcpy(ht, p1.jobmap.data(), p1.jobmap.size() * 4);
  memcpy(ht + p1.jobmap.size() * 4, p1.tiles.data(), p1.tiles.size() * sizeof(Tile));
  MixedBuffers b{};
  b.ctr = static_cast<long long *>(sl.ctr.p);
  b.info_a = static_cast<SInfo *>(sl.info.p);
  b.info_b = static_cast<const SInfo *>(ix.info.p);
  b.tinfo_a = static_cast<float2 *>(sl.tinfo.p);
  b.tinfo_b = static_cast<const float2 *>(ix.tinfo.p);
  for (int d = 0; d < 4; ++d) b.dig_a[d] = static_cast<__nv_bfloat16 *>(sl.dig[d].p);
  for (int d = 0; d < 3; ++d) b.dig_b[d] = static_cast<const __nv_bfloat16 *>(ix.dig[d].p);
  b.pitch_a = b.pitch_b = bk.pitch;
  b.rows_a = blk * kBlockRows;
  b.rows_b = ix.rows;
  b.jobs = static_cast<Job *>(sl.jobs.p);
  b.jobmap = static_cast<int *>(sl.jobmap.p);
  b.tiles = static_cast<Tile *>(sl.tiles.p);
  b.flags = static_cast<unsigned long long *>(sl.flags.p);
  b.flag_cap = kServerFlagCap;
  b.sc = static_cast<DevScalars *>(sl.scal.p);
  CUtensorMap tm[7];
  if (!encode_maps(s->encode, b, tm).empty()) return false;
  uint32_t *prerep = static_cast<uint32_t *>(sl.prerep.p);
  // the pre-screen runs on the slot's high-priority stream (its blocks go
  // ahead of other batches' screens), after the coordinates' copy
  cudaStream_t ps = sl.pst;
  if (cudaEventRecord(sl.pev, sl.st) != cudaSuccess || cudaStreamWaitEvent(ps, sl.pev, 0) != cudaSuccess) return false;
  uint32_t *thr = static_cast<uint32_t *>(sl.thr.p);
  if (cudaMemcpyAsync(b.jobmap, ht, p1.jobmap.size() * 4, cudaMemcpyHostToDevice, ps) != cudaSuccess ||
      cudaMemcpyAsync(b.tiles, ht + p1.jobmap.size() * 4, p1.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice,
                      ps) != cudaSuccess ||
      enqueue_mixed(p1, b, static_cast<const Job *>(sl.hjobs.p), tm, s->num_sms, ps, nullptr, false) !=
          cudaSuccess ||
      launch_screen_select(pre, rows, H, ldh, k, kCandCap, static_cast<uint32_t *>(sl.hist.p), thr,
                           static_cast<int *>(sl.cand_j.p), static_cast<int *>(sl.cand_n.p), ps) != cudaSuccess)
    return false;
  k_gather_cols<<<dim3((unsigned)((R + 127) / 128), (unsigned)rows), 128, 0, ps>>>(
      pre, ldh, static_cast<const int *>(ix.rep_slot.p), R, rows, prerep);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(sl.hpre.p, prerep, (size_t)rows * R * 4, cudaMemcpyDeviceToHost, ps) != cudaSuccess ||
      cudaMemcpyAsync(static_cast<uint32_t *>(sl.hpre.p) + (size_t)rows * R, thr, (size_t)rows * 4,
                      cudaMemcpyDeviceToHost, ps) != cudaSuccess ||
      cudaMemcpyAsync(sl.hback.p, b.jobs, (size_t)nj * sizeof(Job), cudaMemcpyDeviceToHost, ps) != cudaSuccess ||
      cudaMemcpyAsync(sl.hsc.p, b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ps) != cudaSuccess ||
      cudaStreamSynchronize(ps) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const Job *back = static_cast<const Job *>(sl.hback.p);
  for (int j = 0; j < nj; ++j) {
    std::string msg;
    if (collect_errors(*static_cast<const DevScalars *>(sl.hsc.p), back + j, 1, msg) != BS_OK) return false;
  }
  // per row: nearest representative and the bound of its k-th nearest
  static const std::vector<float> half_table = [] {
    std::vector<float> t(65536);
    for (uint32_t h = 0; h < 65536; ++h) t[h] = half_bits_to_float(h);
    return t;
  }();
  const float *ht16 = half_table.data();
  const uint32_t *hp = static_cast<const uint32_t *>(sl.hpre.p);
  const uint32_t *hthr = hp + (size_t)rows * R;
  std::vector<float> lo((size_t)rows * R), test(rows);
  std::vector<int> nearest(rows);
  for (int64_t r = 0; r < rows; ++r) {
    float best = INFINITY;
    int arg = 0;
    for (int c = 0; c < R; ++c) {
      const float l = ht16[hp[r * R + c] & 0xffffu];
      lo[(size_t)r * R + c] = l;
      if (l < best) best = l, arg = c;
    }
    // the threshold is the top edge of the bin of the k-th smallest upper
    // bracket over the heads (0xffff: fewer than k): T >= the k-th nearest
    const float t = hthr[r] >= 0xffffu ? INFINITY : ht16[hthr[r] & 0xffffu];
    test[r] = t + 2.f * s->tol * 1.001f;
    nearest[r] = arg;
  }
  order.assign(nj, {});
  for (int j = 0; j < nj; ++j) {
    const int64_t q = base.jobs[j].n;
    std::vector<int> &o = order[j];
    o.resize(q);
    for (int64_t t = 0; t < q; ++t) o[t] = (int)t;
    const int64_t r0 = sl.row0[j];
    std::stable_sort(o.begin(), o.end(), [&](int a, int c) { return nearest[r0 + a] < nearest[r0 + c]; });
  }
  // per query block: need_c = min over its queries of lo - T; library block
  // b is needed unless every cluster in it has largest bound d < need_c
  const int64_t nbb = (bk.n + kBStructs - 1) / kBStructs;
  need.assign(blk, {});
  std::vector<float> nc(R);
  for (int j = 0; j < nj; ++j) {
    const int64_t q = base.jobs[j].n, b0 = base.jobs[j].first_a / kBlockStructs;
    for (int64_t I = 0; I * kBlockStructs < q; ++I) {
      std::fill(nc.begin(), nc.end(), INFINITY);
      for (int64_t u = I * kBlockStructs; u < std::min<int64_t>(q, (I + 1) * kBlockStructs); ++u) {
        const int64_t r = sl.row0[j] + order[j][u];
        const float tr = test[r];
        const float *lr = &lo[(size_t)r * R];
        for (int c = 0; c < R; ++c) nc[c] = std::min(nc[c], lr[c] - tr);
      }
      std::vector<int64_t> &v = need[b0 + I];
      for (int64_t lb = 0; lb < nbb; ++lb) {
        const int a0 = ix.c0[lb], a1 = ix.c1[lb];
        if (a0 < 0 || ix.d0[lb] >= nc[a0] || (a1 >= 0 && ix.d1[lb] >= nc[a1])) v.push_back(lb);
      }
    }
  }
  return true;
}

// Enqueues a query batch on the slot.  screen: the two-stage top-k (bounds
// from the leading levels on the tensor cores, then the certified crmsd of
// each row's candidates); otherwise every pair is certified densely.  On an
// indexed bucket a screen first runs against the representatives
// (index_prescreen) and then only on the library blocks that can hold a
// query's nearest; each request's queries are then processed in the order of
// their nearest representative and their results mapped back (row_of).
bs_status launch_query_batch(bs_server *s, Slot &sl, bool screen) {
  const Bucket &bk = s->buckets[sl.bucket];
  const int L = bk.L, k = s->top_k;
  const int nj = (int)sl.reqs.size();
  // host plan: one rectangular job per request
  Plan plan;
  plan.pitch = bk.pitch;
  sl.row0.assign(nj, 0);
  int64_t blk = 0, rows = 0;
  size_t xyz_off = 0;
  std::vector<size_t> xoff(nj);
  for (int j = 0; j < nj; ++j) {
    const Request *r = sl.reqs[j];
    sl.row0[j] = rows;
    xoff[j] = xyz_off;
    xyz_off += (size_t)r->q * L * 3;
    const int64_t nb = blocks_for(r->q);
    for (int64_t b = 0; b < nb; ++b) plan.jobmap.push_back(j);
    Job jb{};
    jb.n = r->q;
    jb.first_a = blk * kBlockStructs;
    jb.first_b = 0;
    jb.n_b = bk.n;
    jb.L = L;
    jb.lp = bk.lp;
    jb.mode = 1;
    jb.fixed_scale = 1;
    jb.scale_min = bk.scale_exp;
    jb.tol = s->tol;
    for (int d = 0; d < 3; ++d) jb.norm_b[d] = bk.norm_b[d];
    jb.qres_b = bk.qres;
    jb.screen = screen ? 1 : 0;
    plan.jobs.push_back(jb);
    blk += nb;
    rows += r->q;
  }
  const int64_t nbb = (bk.n + kBStructs - 1) / kBStructs;
  const int nk16 = bk.lp / 16;
  plan.strips = screen && s->precision == BS_PRECISION_MIXED && nk16 <= screen_strip_max_nk16();
  plan.nblocks = blk;
  sl.rows = rows;
  sl.njobs = nj;
  sl.screen = screen && s->precision == BS_PRECISION_MIXED;
  sl.row_of.clear();
  const int64_t ns = blk * kBlockStructs, drows = blk * kBlockRows;
  const bool plain = s->precision == BS_PRECISION_PLAIN64;
  // screen batches: one packed bracket word per pair, rows padded to 4 words
  const int64_t ld = sl.screen ? ((bk.n + 3) & ~int64_t(3)) : bk.n;
  // tiles column block by column block: the persistent blocks sweep the
  // library once, each library block read from HBM once and reused from L2
  // by every query block of the batch.  Screens of chains the strip kernel
  // takes run as strips: a query block against a run of library blocks,
  // the query block's digits resident in shared memory for the run; runs
  // sized for about a dozen per block of the grid.
  batch_tiles(s, plan, blk, nbb, nk16, plan.strips, nullptr, plan.tiles);
  bool ok = sv_ensure(s, sl, sl.xyz, xyz_off * 8) && sv_ensure(s, sl, sl.dense, (size_t)rows * ld * 4) &&
            sv_ensure(s, sl, sl.topi, (size_t)rows * k * 8) && sv_ensure(s, sl, sl.topv, (size_t)rows * k * 4) &&
            sv_ensure(s, sl, sl.scal, sizeof(DevScalars)) && host_ensure(sl, sl.hxyz, xyz_off * 8) &&
            host_ensure(sl, sl.htopi, (size_t)rows * k * 8) && host_ensure(sl, sl.htopv, (size_t)rows * k * 4) &&
            host_ensure(sl, sl.hsc, sizeof(DevScalars));
  if (plain) {
    ok = ok && sv_ensure(s, sl, sl.y, (size_t)rows * 3 * bk.lp * 8) && sv_ensure(s, sl, sl.g, (size_t)rows * 8) &&
         sv_ensure(s, sl, sl.ctrd, (size_t)rows * 24);
  } else {
    ok = ok && sv_ensure(s, sl, sl.ctr, (size_t)ns * 24) && sv_ensure(s, sl, sl.info, (size_t)ns * 16) &&
         sv_ensure(s, sl, sl.jobs, (size_t)nj * sizeof(Job)) && sv_ensure(s, sl, sl.jobmap, plan.jobmap.size() * 4) &&
         sv_ensure(s, sl, sl.tiles, plan.tiles.size() * sizeof(Tile)) && sv_ensure(s, sl, sl.flags, kServerFlagCap * 8) &&
         host_ensure(sl, sl.hjobs, (size_t)nj * sizeof(Job)) && host_ensure(sl, sl.hback, (size_t)nj * sizeof(Job)) &&
         host_ensure(sl, sl.htab, plan.jobmap.size() * 4 + plan.tiles.size() * sizeof(Tile) + (size_t)rows * 12 + 16);
    for (int d = 0; d < 4 && ok; ++d) ok = sv_ensure(s, sl, sl.dig[d], (size_t)drows * bk.pitch * 2);
    if (sl.screen)
      ok = ok && sv_ensure(s, sl, sl.tinfo, (size_t)ns * 8) && sv_ensure(s, sl, sl.hist, (size_t)rows * kScreenBins * 4) &&
           sv_ensure(s, sl, sl.thr, (size_t)rows * 4) &&
           sv_ensure(s, sl, sl.cand_j, (size_t)rows * kCandCap * 4) &&
           sv_ensure(s, sl, sl.cand_n, (size_t)rows * 4) && sv_ensure(s, sl, sl.cand_v, (size_t)rows * kCandCap * 4) &&
           sv_ensure(s, sl, sl.rowtab, (size_t)rows * 12 + 8) && host_ensure(sl, sl.hcand_n, (size_t)rows * 4);
  }
  if (!ok) return BS_ERR_OOM;
  // coordinates in
  double *hx = static_cast<double *>(sl.hxyz.p);
  for (int j = 0; j < nj; ++j) memcpy(hx + xoff[j], sl.reqs[j]->xyz.data(), sl.reqs[j]->xyz.size() * 8);
  double *dx = static_cast<double *>(sl.xyz.p);
  if (cudaMemcpyAsync(dx, hx, xyz_off * 8, cudaMemcpyHostToDevice, sl.st) != cudaSuccess) return BS_ERR_CUDA;
  bool pruned = false;
  std::vector<std::vector<int64_t>> need;  // pruned screens: library blocks per query block
  if (sl.screen && bk.indexed) {
    std::vector<std::vector<int>> order;
    const bool usable = index_prescreen(s, sl, plan, blk, rows, dx, xoff, order, need);
    if (!usable) cudaStreamSynchronize(sl.pst);  // nothing of the pre-screen may still run
    if (usable) {
      pruned = true;
      // each request's queries in the order of their nearest representative
      sl.row_of.assign(rows, 0);
      for (int j = 0; j < nj; ++j) {
        const size_t one = (size_t)L * 3;
        const double *src = sl.reqs[j]->xyz.data();
        for (size_t u = 0; u < order[j].size(); ++u) {
          memcpy(hx + xoff[j] + u * one, src + (size_t)order[j][u] * one, one * 8);
          sl.row_of[sl.row0[j] + order[j][u]] = sl.row0[j] + (int64_t)u;
        }
      }
      if (cudaMemcpyAsync(dx, hx, xyz_off * 8, cudaMemcpyHostToDevice, sl.st) != cudaSuccess) return BS_ERR_CUDA;
      batch_tiles(s, plan, blk, nbb, nk16, plan.strips, &need, plan.tiles);
      if (!sv_ensure(s, sl, sl.tiles, plan.tiles.size() * sizeof(Tile)) ||
          !host_ensure(sl, sl.htab, plan.jobmap.size() * 4 + plan.tiles.size() * sizeof(Tile) + (size_t)rows * 12 + 16))
        return BS_ERR_OOM;
    }
  }
  float *dense = static_cast<float *>(sl.dense.p);
  if (plain) {
    if (cudaMemsetAsync(sl.scal.p, 0, sizeof(DevScalars), sl.st) != cudaSuccess) return BS_ERR_CUDA;
    for (int j = 0; j < nj; ++j) {
      const Request *r = sl.reqs[j];
      OutDesc od{dense + sl.row0[j] * bk.n, r->q, bk.n, kLayoutRect, 1};
      if (launch_prep_plain(dx + xoff[j], r->q, L, bk.lp, static_cast<double *>(sl.ctrd.p),
                            static_cast<double *>(sl.y.p), static_cast<double *>(sl.g.p),
                            &static_cast<DevScalars *>(sl.scal.p)->err, sl.st) != cudaSuccess ||
          launch_plain64_rect(static_cast<const double *>(sl.y.p), static_cast<const double *>(sl.g.p), r->q,
                              static_cast<const double *>(bk.y.p), static_cast<const double *>(bk.g.p), bk.n, L,
                              bk.lp, od, sl.st) != cudaSuccess)
        return BS_ERR_CUDA;
    }
  } else {
    // pruned screens: the selection reads the screened segments only
    std::vector<SelSeg> segs;
    if (pruned) {
      const int64_t chunk = screen_select_chunk();
      for (int j = 0; j < nj; ++j) {
        const int64_t q = plan.jobs[j].n, b0 = plan.jobs[j].first_a / kBlockStructs;
        for (int64_t I = 0; I * kBlockStructs < q; ++I) {
          const int64_t r0 = sl.row0[j] + I * kBlockStructs;
          const int nr = (int)std::min<int64_t>(kBlockStructs, q - I * kBlockStructs);
          const std::vector<int64_t> &v = need[b0 + I];
          for (size_t a = 0; a < v.size();) {
            size_t e = a + 1;
            while (e < v.size() && v[e] == v[e - 1] + 1) ++e;
            const int64_t c1 = std::min<int64_t>(bk.n, v[e - 1] * kBStructs + kBStructs);
            for (int64_t c = v[a] * kBStructs; c < c1; c += chunk)
              segs.push_back(SelSeg{r0, nr, 0, c, std::min(c + chunk, c1)});
            a = e;
          }
        }
      }
      if (!sv_ensure(s, sl, sl.segs, segs.size() * sizeof(SelSeg)) || !host_ensure(sl, sl.hsegs, segs.size() * sizeof(SelSeg)))
        return BS_ERR_OOM;
      memcpy(sl.hsegs.p, segs.data(), segs.size() * sizeof(SelSeg));
      if (cudaMemcpyAsync(sl.segs.p, sl.hsegs.p, segs.size() * sizeof(SelSeg), cudaMemcpyHostToDevice, sl.st) !=
          cudaSuccess)
        return BS_ERR_CUDA;
    }
    if (sl.screen) {
      int64_t t = 0;
      for (const Tile &tl : plan.tiles) t += plan.strips ? (tl.shape >> 16) : 1;
      s->screened += t * kBlockStructs * kBStructs;
    }
    for (int j = 0; j < nj; ++j) plan.jobs[j].xyz = dx + xoff[j];
    for (int j = 0; j < nj; ++j) plan.jobs[j].out = OutDesc{dense + sl.row0[j] * ld, sl.reqs[j]->q, ld, kLayoutRect, 1};
    memcpy(sl.hjobs.p, plan.jobs.data(), (size_t)nj * sizeof(Job));
    char *ht = static_cast<char *>(sl.htab.p);
    memcpy(ht, plan.jobmap.data(), plan.jobmap.size() * 4);
    memcpy(ht + plan.jobmap.size() * 4, plan.tiles.data(), plan.tiles.size() * sizeof(Tile));
    MixedBuffers b{};
    b.ctr = static_cast<long long *>(sl.ctr.p);
    b.info_a = static_cast<SInfo *>(sl.info.p);
    b.info_b = static_cast<const SInfo *>(bk.info.p);
    if (sl.screen) {
      b.tinfo_a = static_cast<float2 *>(sl.tinfo.p);
      b.tinfo_b = static_cast<const float2 *>(bk.tinfo.p);
    }
    for (int d = 0; d < 4; ++d) b.dig_a[d] = static_cast<__nv_bfloat16 *>(sl.dig[d].p);
    for (int d = 0; d < 3; ++d) b.dig_b[d] = static_cast<const __nv_bfloat16 *>(bk.dig[d].p);
    b.pitch_a = bk.pitch;
    b.pitch_b = bk.pitch;
    b.rows_a = drows;
    b.rows_b = bk.rows;
    b.jobs = static_cast<Job *>(sl.jobs.p);
    b.jobmap = static_cast<int *>(sl.jobmap.p);
    b.tiles = static_cast<Tile *>(sl.tiles.p);
    b.flags = static_cast<unsigned long long *>(sl.flags.p);
    b.flag_cap = kServerFlagCap;
    b.sc = static_cast<DevScalars *>(sl.scal.p);
    CUtensorMap tm[7];
    if (!encode_maps(s->encode, b, tm).empty()) return BS_ERR_CUDA;
    if (cudaMemcpyAsync(b.jobmap, ht, plan.jobmap.size() * 4, cudaMemcpyHostToDevice, sl.st) != cudaSuccess ||
        cudaMemcpyAsync(b.tiles, ht + plan.jobmap.size() * 4, plan.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice,
                        sl.st) != cudaSuccess ||
        enqueue_mixed(plan, b, static_cast<const Job *>(sl.hjobs.p), tm, s->num_sms, sl.st, nullptr, false) !=
            cudaSuccess ||
        cudaMemcpyAsync(sl.hback.p, b.jobs, (size_t)nj * sizeof(Job), cudaMemcpyDeviceToHost, sl.st) != cudaSuccess)
      return BS_ERR_CUDA;
    if (sl.screen) {
      // per row: job and global A structure, for the certified candidates
      // (int job[rows] padded to 8 bytes, then int64 structure[rows])
      const size_t jbytes = ((size_t)rows * 4 + 7) & ~size_t(7);
      char *rt = ht + plan.jobmap.size() * 4 + plan.tiles.size() * sizeof(Tile);
      rt = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(rt) + 7) & ~uintptr_t(7));
      int *rjob = reinterpret_cast<int *>(rt);
      int64_t *rig = reinterpret_cast<int64_t *>(rt + jbytes);
      for (int j = 0; j < nj; ++j)
        for (int64_t t = 0; t < sl.reqs[j]->q; ++t) {
          rjob[sl.row0[j] + t] = j;
          rig[sl.row0[j] + t] = plan.jobs[j].first_a + t;
        }
      int *drjob = static_cast<int *>(sl.rowtab.p);
      const int64_t *drig = reinterpret_cast<const int64_t *>(static_cast<char *>(sl.rowtab.p) + jbytes);
      const int *cj = static_cast<const int *>(sl.cand_j.p);
      const int *cn = static_cast<const int *>(sl.cand_n.p);
      if (cudaMemcpyAsync(drjob, rt, jbytes + (size_t)rows * 8, cudaMemcpyHostToDevice, sl.st) != cudaSuccess ||
          (pruned ? launch_screen_select_seg(reinterpret_cast<const uint32_t *>(dense), rows, ld, k, kCandCap,
                                             static_cast<const SelSeg *>(sl.segs.p), (int64_t)segs.size(),
                                             kBlockStructs, static_cast<uint32_t *>(sl.hist.p),
                                             static_cast<uint32_t *>(sl.thr.p), static_cast<int *>(sl.cand_j.p),
                                             static_cast<int *>(sl.cand_n.p), sl.st)
                  : launch_screen_select(reinterpret_cast<const uint32_t *>(dense), rows, bk.n, ld, k, kCandCap,
                                         static_cast<uint32_t *>(sl.hist.p), static_cast<uint32_t *>(sl.thr.p),
                                         static_cast<int *>(sl.cand_j.p), static_cast<int *>(sl.cand_n.p),
                                         sl.st)) != cudaSuccess ||
          launch_exact_candidates(DigitsView{b.dig_a[0], b.dig_a[1], b.dig_a[2], b.pitch_a},
                                  DigitsView{b.dig_b[0], b.dig_b[1], b.dig_b[2], b.pitch_b}, b.info_a, b.info_b, b.jobs,
                                  drjob, drig, rows, cj, cn, kCandCap, static_cast<float *>(sl.cand_v.p),
                                  sl.st) != cudaSuccess ||
          launch_topk_rows(static_cast<const float *>(sl.cand_v.p), rows, cn, kCandCap, k, cj, bk_perm(bk),
                           static_cast<int64_t *>(sl.topi.p), static_cast<float *>(sl.topv.p), sl.st) != cudaSuccess ||
          cudaMemcpyAsync(sl.hcand_n.p, cn, (size_t)rows * 4, cudaMemcpyDeviceToHost, sl.st) != cudaSuccess)
        return BS_ERR_CUDA;
    }
  }
  if ((!sl.screen && launch_topk(dense, rows, bk.n, bk.n, k, bk_perm(bk), static_cast<int64_t *>(sl.topi.p),
                                 static_cast<float *>(sl.topv.p), sl.st) != cudaSuccess) ||
      cudaMemcpyAsync(sl.htopi.p, sl.topi.p, (size_t)rows * k * 8, cudaMemcpyDeviceToHost, sl.st) != cudaSuccess ||
      cudaMemcpyAsync(sl.htopv.p, sl.topv.p, (size_t)rows * k * 4, cudaMemcpyDeviceToHost, sl.st) != cudaSuccess ||
      cudaMemcpyAsync(sl.hsc.p, sl.scal.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, sl.st) != cudaSuccess ||
      cudaEventRecord(sl.ev, sl.st) != cudaSuccess)
    return BS_ERR_CUDA;
  return BS_OK;
}

// A query outside its bucket's grid: the plain FP64 path, synchronously on
// the slot's stream, into the slot's dense rows of that job.
bs_status plain_fallback(bs_server *s, Slot &sl, int j) {
  const Bucket &bk = s->buckets[sl.bucket];
  const Request *r = sl.reqs[j];
  const int k = s->top_k;
  if (!sv_ensure(s, sl, sl.y, (size_t)r->q * 3 * bk.lp * 8) || !sv_ensure(s, sl, sl.g, (size_t)r->q * 8) ||
      !sv_ensure(s, sl, sl.ctrd, (size_t)r->q * 24) || !sv_ensure(s, sl, sl.xyz, r->xyz.size() * 8))
    return BS_ERR_OOM;
  float *dense = static_cast<float *>(sl.dense.p) + sl.row0[j] * bk.n;
  OutDesc od{dense, r->q, bk.n, kLayoutRect, 1};
  DevScalars *sc = static_cast<DevScalars *>(sl.scal.p);
  if (cudaMemsetAsync(sc, 0, sizeof(DevScalars), sl.st) != cudaSuccess ||
      cudaMemcpyAsync(sl.xyz.p, r->xyz.data(), r->xyz.size() * 8, cudaMemcpyHostToDevice, sl.st) != cudaSuccess ||
      launch_prep_plain(static_cast<const double *>(sl.xyz.p), r->q, bk.L, bk.lp, static_cast<double *>(sl.ctrd.p),
                        static_cast<double *>(sl.y.p), static_cast<double *>(sl.g.p), &sc->err, sl.st) != cudaSuccess ||
      launch_plain64_rect(static_cast<const double *>(sl.y.p), static_cast<const double *>(sl.g.p), r->q,
                          static_cast<const double *>(bk.y.p), static_cast<const double *>(bk.g.p), bk.n, bk.L, bk.lp,
                          od, sl.st) != cudaSuccess ||
      launch_topk(dense, r->q, bk.n, bk.n, k, bk_perm(bk), static_cast<int64_t *>(sl.topi.p) + sl.row0[j] * k,
                  static_cast<float *>(sl.topv.p) + sl.row0[j] * k, sl.st) != cudaSuccess ||
      cudaMemcpyAsync(static_cast<int64_t *>(sl.htopi.p) + sl.row0[j] * k,
                      static_cast<int64_t *>(sl.topi.p) + sl.row0[j] * k, (size_t)r->q * k * 8, cudaMemcpyDeviceToHost,
                      sl.st) != cudaSuccess ||
      cudaMemcpyAsync(static_cast<float *>(sl.htopv.p) + sl.row0[j] * k,
                      static_cast<float *>(sl.topv.p) + sl.row0[j] * k, (size_t)r->q * k * 4, cudaMemcpyDeviceToHost,
                      sl.st) != cudaSuccess ||
      cudaMemcpyAsync(sl.hsc.p, sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, sl.st) != cudaSuccess ||
      cudaStreamSynchronize(sl.st) != cudaSuccess)
    return BS_ERR_CUDA;
  if (static_cast<DevScalars *>(sl.hsc.p)->err & kErrNonFinite) return BS_ERR_NONFINITE;
  return BS_OK;
}

bs_status launch_cluster_batch(bs_server *s, Slot &sl) {
  Request *r = sl.reqs[0];
  const int64_t n = r->q;
  const size_t tri = (size_t)(n * (n - 1) / 2);
  if (!sv_ensure(s, sl, sl.xyz, r->xyz.size() * 8) || !sv_ensure(s, sl, sl.dense, tri * 4) ||
      !host_ensure(sl, sl.htri, tri * 4) || !host_ensure(sl, sl.hxyz, r->xyz.size() * 8) ||
      !sv_ensure(s, sl, sl.scal, sizeof(DevScalars)) || !host_ensure(sl, sl.hsc, sizeof(DevScalars)))
    return BS_ERR_OOM;
  memcpy(sl.hxyz.p, r->xyz.data(), r->xyz.size() * 8);
  if (cudaMemcpyAsync(sl.xyz.p, sl.hxyz.p, r->xyz.size() * 8, cudaMemcpyHostToDevice, sl.st) != cudaSuccess)
    return BS_ERR_CUDA;
  std::vector<JobSpec> specs{JobSpec{static_cast<const double *>(sl.xyz.p), n, r->L,
                                     OutDesc{sl.dense.p, n, n, kLayoutTriangle, 1}}};
  if (s->precision == BS_PRECISION_PLAIN64) {
    const int lp = lp_for(r->L);
    if (!sv_ensure(s, sl, sl.y, (size_t)n * 3 * lp * 8) || !sv_ensure(s, sl, sl.g, (size_t)n * 8) ||
        !sv_ensure(s, sl, sl.ctrd, (size_t)n * 24))
      return BS_ERR_OOM;
    DevScalars *sc = static_cast<DevScalars *>(sl.scal.p);
    if (cudaMemsetAsync(sc, 0, sizeof(DevScalars), sl.st) != cudaSuccess ||
        launch_prep_plain(specs[0].xyz, n, r->L, lp, static_cast<double *>(sl.ctrd.p), static_cast<double *>(sl.y.p),
                          static_cast<double *>(sl.g.p), &sc->err, sl.st) != cudaSuccess ||
        launch_plain64_all(static_cast<const double *>(sl.y.p), static_cast<const double *>(sl.g.p), n, r->L, lp,
                           specs[0].out, sl.st) != cudaSuccess)
      return BS_ERR_CUDA;
    sl.njobs = 0;
  } else {
    Plan plan;
    if (!make_symmetric_plan(specs, s->tol, true, plan).empty()) return BS_ERR_UNSUPPORTED;
    const int64_t ns = plan.nblocks * kBlockStructs, drows = plan.nblocks * kBlockRows;
    bool ok = sv_ensure(s, sl, sl.ctr, (size_t)ns * 24) && sv_ensure(s, sl, sl.info, (size_t)ns * 16) &&
              sv_ensure(s, sl, sl.jobs, sizeof(Job)) && sv_ensure(s, sl, sl.jobmap, plan.jobmap.size() * 4) &&
              sv_ensure(s, sl, sl.tiles, plan.tiles.size() * sizeof(Tile)) && sv_ensure(s, sl, sl.flags, kServerFlagCap * 8) &&
              host_ensure(sl, sl.hjobs, sizeof(Job)) && host_ensure(sl, sl.hback, sizeof(Job)) &&
              host_ensure(sl, sl.htab, plan.jobmap.size() * 4 + plan.tiles.size() * sizeof(Tile));
    for (int d = 0; d < 4 && ok; ++d) ok = sv_ensure(s, sl, sl.dig[d], (size_t)drows * plan.pitch * 2);
    if (!ok) return BS_ERR_OOM;
    MixedBuffers b{};
    b.ctr = static_cast<long long *>(sl.ctr.p);
    b.info_a = static_cast<SInfo *>(sl.info.p);
    b.info_b = b.info_a;
    for (int d = 0; d < 4; ++d) b.dig_a[d] = static_cast<__nv_bfloat16 *>(sl.dig[d].p);
    for (int d = 0; d < 3; ++d) b.dig_b[d] = b.dig_a[d];
    b.pitch_a = b.pitch_b = plan.pitch;
    b.rows_a = b.rows_b = drows;
    b.jobs = static_cast<Job *>(sl.jobs.p);
    b.jobmap = static_cast<int *>(sl.jobmap.p);
    b.tiles = static_cast<Tile *>(sl.tiles.p);
    b.flags = static_cast<unsigned long long *>(sl.flags.p);
    b.flag_cap = kServerFlagCap;
    b.sc = static_cast<DevScalars *>(sl.scal.p);
    memcpy(sl.hjobs.p, plan.jobs.data(), sizeof(Job));
    char *ht = static_cast<char *>(sl.htab.p);
    memcpy(ht, plan.jobmap.data(), plan.jobmap.size() * 4);
    memcpy(ht + plan.jobmap.size() * 4, plan.tiles.data(), plan.tiles.size() * sizeof(Tile));
    CUtensorMap tm[7];
    if (!encode_maps(s->encode, b, tm).empty()) return BS_ERR_CUDA;
    if (cudaMemcpyAsync(b.jobmap, ht, plan.jobmap.size() * 4, cudaMemcpyHostToDevice, sl.st) != cudaSuccess ||
        cudaMemcpyAsync(b.tiles, ht + plan.jobmap.size() * 4, plan.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice,
                        sl.st) != cudaSuccess ||
        enqueue_mixed(plan, b, static_cast<const Job *>(sl.hjobs.p), tm, s->num_sms, sl.st, nullptr, false) !=
            cudaSuccess ||
        cudaMemcpyAsync(sl.hback.p, b.jobs, sizeof(Job), cudaMemcpyDeviceToHost, sl.st) != cudaSuccess)
      return BS_ERR_CUDA;
    sl.njobs = 1;
  }
  if (cudaMemcpyAsync(sl.htri.p, sl.dense.p, tri * 4, cudaMemcpyDeviceToHost, sl.st) != cudaSuccess ||
      cudaMemcpyAsync(sl.hsc.p, sl.scal.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, sl.st) != cudaSuccess ||
      cudaEventRecord(sl.ev, sl.st) != cudaSuccess)
    return BS_ERR_CUDA;
  return BS_OK;
}

// Sizes every slot's buffers for a full batch of each bucket before the
// server takes requests, so that no buffer grows while requests wait.  Slot
// 0 runs one batch of max_rows library structures (requests of 64) per
// bucket and the other slots take the same capacities.  Buckets whose full
// batch the budget cannot hold in every slot are skipped (their buffers grow
// on demand), and so is the plain FP64 path (its batches are slow).
bs_status reserve_slots(bs_server *s, const bs_server_config *cfg) {
  if (s->precision != BS_PRECISION_MIXED || s->slots.empty()) return BS_OK;
  Slot &s0 = *s->slots[0];
  const size_t nslots = s->slots.size();
  for (int b = 0; b < (int)s->buckets.size(); ++b) {
    const Bucket &bk = s->buckets[b];
    const int L = bk.L;
    const size_t one = (size_t)L * 3;
    const int64_t take = std::min<int64_t>(bk.n, 64);
    std::vector<double> src(take * one);
    if (is_device_ptr(cfg->bucket_xyz[b])) {
      if (cudaMemcpy(src.data(), cfg->bucket_xyz[b], src.size() * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return BS_ERR_CUDA;
    } else {
      memcpy(src.data(), cfg->bucket_xyz[b], src.size() * 8);
    }
    std::vector<std::unique_ptr<Request>> reqs;
    std::vector<Request *> batch;
    for (int64_t rows = 0; rows < s->max_rows;) {
      auto r = std::make_unique<Request>();
      r->bucket = b;
      r->L = L;
      r->q = std::min<int64_t>(64, s->max_rows - rows);
      r->xyz.resize(r->q * one);
      for (int64_t t = 0; t < r->q; ++t)
        memcpy(r->xyz.data() + t * one, src.data() + ((rows + t) % take) * one, one * 8);
      rows += r->q;
      batch.push_back(r.get());
      reqs.push_back(std::move(r));
    }
    if (s->used + batch_bytes(s, batch) * 5 / 4 * nslots > s->budget) continue;
    s0.reqs = batch;
    s0.kind = 0;
    s0.bucket = b;
    bs_status st = launch_query_batch(s, s0, true);
    if (st == BS_OK && cudaEventSynchronize(s0.ev) != cudaSuccess) st = BS_ERR_CUDA;
    s0.reqs.clear();
    if (st) {
      cudaGetLastError();
      cudaStreamSynchronize(s0.st);
      return st;
    }
  }
  std::vector<DevBuf *> d0;
  std::vector<HostBuf *> h0;
  each_dev(s0, [&](DevBuf &x) { d0.push_back(&x); });
  each_host(s0, [&](HostBuf &x) { h0.push_back(&x); });
  for (size_t i = 1; i < nslots; ++i) {
    Slot &o = *s->slots[i];
    size_t k = 0;
    bool ok = true;
    each_dev(o, [&](DevBuf &x) {
      const size_t cap = d0[k++]->cap;
      if (ok && cap > x.cap) ok = sv_ensure(s, o, x, cap * 4 / 5);
    });
    k = 0;
    each_host(o, [&](HostBuf &x) {
      const size_t cap = h0[k++]->cap;
      if (ok && cap > x.cap) ok = host_ensure(o, x, cap * 4 / 5);
    });
    if (!ok) return BS_ERR_OOM;
  }
  s->screened = 0;
  return BS_OK;
}

void complete(bs_server *s, Request *r, bs_status st, const std::string &msg) {
  r->status = st;
  r->err = msg;
  r->t_done = Clock::now();
  r->done = true;
  const double ms = ms_between(r->t_submit, r->t_done);
  if (!s->trace_path.empty()) {
    char line[160];
    snprintf(line, sizeof line, "R,%lld,%d,%d,%lld,%.3f,%.3f,%lld,%d", (long long)r->id, r->kind, r->bucket,
             (long long)r->q, ms_between(s->t0, r->t_submit), ms_between(s->t0, r->t_done), (long long)r->batch,
             (int)st);
    s->trace.emplace_back(line);
  }
  if (st == BS_OK) {
    if (r->kind == 0) {
      s->lat.push_back(ms);
      ++s->qdone;
    } else {
      s->clat.push_back(ms);
      ++s->cdone;
    }
    s->pairs += r->pairs;
  }
  s->cv_done.notify_all();
}

// ------------------------------------------------------------ index
constexpr int64_t kIndexPerRep = 512;  // structures per representative
constexpr int64_t kIndexMinDefault = 16384;  // buckets indexed by default
constexpr int kIndexMaxReps = 256;

struct DigitPtrs {
  const __nv_bfloat16 *src[4];
  __nv_bfloat16 *dst[4];
};

// Structure r of a set (bucket position pos[r]): its three digit rows of
// each digit matrix, its SInfo and its screen data, into slot r of a set
// laid out like a bucket (one block per structure).
__global__ void k_gather_reps(DigitPtrs d, int pitch, const int64_t *__restrict__ pos, int R,
                              const SInfo *__restrict__ info_src, SInfo *__restrict__ info_dst,
                              const float2 *__restrict__ t_src, float2 *__restrict__ t_dst) {
  const int r = blockIdx.x;
  if (r >= R) return;
  const int64_t p = pos[r];
  for (int c = 0; c < 3; ++c) {
    const int64_t rs = digit_row(p, c) * pitch, rd = digit_row(r, c) * pitch;
    for (int m = 0; m < 4; ++m)
      for (int k = threadIdx.x; k < pitch; k += blockDim.x) d.dst[m][rd + k] = d.src[m][rs + k];
  }
  if (threadIdx.x == 0) {
    info_dst[r] = info_src[p];
    t_dst[r] = t_src[p];
  }
}

void free_bucket(Bucket &bk) {
  for (DevBuf *d : {&bk.dig[0], &bk.dig[1], &bk.dig[2], &bk.dig[3], &bk.info, &bk.tinfo, &bk.y, &bk.g, &bk.ix.dig[0],
                    &bk.ix.dig[1], &bk.ix.dig[2], &bk.ix.dig[3], &bk.ix.info, &bk.ix.tinfo, &bk.ix.perm,
                    &bk.ix.rep_slot}) {
    if (d->p) cudaFree(d->p);
    d->p = nullptr;
    d->cap = 0;
  }
}

// Builds the library index of bucket bi (see Index) from its coordinates in
// library order on the host, and stores the bucket in cluster order.  The
// representatives are every (n / R)-th structure; their exact crmsd to every
// structure comes from the dense certified path on slot 0.
bs_status build_index(bs_server *s, int bi, const double *xyz) {
  Bucket &bk = s->buckets[bi];
  const int64_t n = bk.n;
  const int L = bk.L, k = s->top_k;
  const int R = (int)std::min<int64_t>(kIndexMaxReps, std::max<int64_t>(2, n / kIndexPerRep));
  std::vector<int64_t> rep(R);
  for (int r = 0; r < R; ++r) rep[r] = (int64_t)r * n / R;
  Slot &sl = *s->slots[0];
  sl.bucket = bi;
  sl.kind = 0;
  std::vector<float> dist((size_t)R * n);
  const size_t one = (size_t)L * 3;
  for (int r0 = 0; r0 < R; r0 += 256) {
    const int cnt = std::min(256, R - r0);
    Request rq;
    rq.kind = 0;
    rq.bucket = bi;
    rq.L = L;
    rq.q = cnt;
    rq.xyz.resize(cnt * one);
    for (int u = 0; u < cnt; ++u) memcpy(rq.xyz.data() + u * one, xyz + rep[r0 + u] * one, one * 8);
    sl.reqs.assign(1, &rq);
    bs_status st = launch_query_batch(s, sl, false);
    if (st == BS_OK && cudaStreamSynchronize(sl.st) != cudaSuccess) st = BS_ERR_CUDA;
    std::string msg;
    if (st == BS_OK)
      st = collect_errors(*static_cast<const DevScalars *>(sl.hsc.p), static_cast<const Job *>(sl.hback.p), 1, msg);
    if (st == BS_OK && cudaMemcpy(dist.data() + (size_t)r0 * n, sl.dense.p, (size_t)cnt * n * 4,
                                  cudaMemcpyDeviceToHost) != cudaSuccess)
      st = BS_ERR_CUDA;
    sl.reqs.clear();
    if (st) {
      s->err = "library index: " + (msg.empty() ? std::string("device error") : msg);
      return st;
    }
  }
  // nearest representative and an upper bound of the distance: the values
  // are certified to tol; the margin covers their f32 rounding
  std::vector<int> cl(n);
  std::vector<float> dd(n);
  for (int64_t x = 0; x < n; ++x) {
    int best = 0;
    float v = dist[x];
    for (int r = 1; r < R; ++r)
      if (dist[(size_t)r * n + x] < v) v = dist[(size_t)r * n + x], best = r;
    cl[x] = best;
    dd[x] = v + s->tol * 1.01f + v * 1e-6f;
  }
  std::vector<int64_t> ord(n);
  for (int64_t x = 0; x < n; ++x) ord[x] = x;
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
    return cl[a] != cl[b] ? cl[a] < cl[b] : (dd[a] != dd[b] ? dd[a] < dd[b] : a < b);
  });
  std::vector<int64_t> pos_of(n);
  for (int64_t u = 0; u < n; ++u) pos_of[ord[u]] = u;
  // the bucket again, in cluster order
  std::vector<double> px(n * one);
  for (int64_t u = 0; u < n; ++u) memcpy(px.data() + u * one, xyz + ord[u] * one, one * 8);
  free_bucket(bk);
  bs_status st = build_bucket(s, bk, px.data());
  if (st) return st;
  Index &ix = bk.ix;
  ix = Index{};
  ix.nrep = R;
  // cluster c occupies positions [first[c], first[c + 1])
  std::vector<int64_t> first(R + 1, n);
  for (int64_t u = n - 1; u >= 0; --u) first[cl[ord[u]]] = u;
  for (int r = R - 1; r >= 0; --r)
    if (first[r] == n || first[r] > first[r + 1]) first[r] = first[r + 1];  // empty clusters
  // per library block: its clusters and their largest bounds
  const int64_t nbb = (n + kBStructs - 1) / kBStructs;
  ix.c0.assign(nbb, -1);
  ix.c1.assign(nbb, -1);
  ix.d0.assign(nbb, 0.f);
  ix.d1.assign(nbb, 0.f);
  for (int64_t b = 0; b < nbb; ++b) {
    const int64_t u0 = b * kBStructs, u1 = std::min(n, u0 + kBStructs);
    const int a = cl[ord[u0]], z = cl[ord[u1 - 1]];
    int distinct = 1;
    for (int64_t u = u0 + 1; u < u1; ++u) distinct += cl[ord[u]] != cl[ord[u - 1]];
    if (distinct > 2) continue;  // c0 = -1: always screened
    ix.c0[b] = a;
    ix.c1[b] = z != a ? z : -1;
    for (int64_t u = u0; u < u1; ++u) {
      const int c = cl[ord[u]];
      float &m = c == a ? ix.d0[b] : ix.d1[b];
      m = std::max(m, dd[ord[u]]);
    }
  }
  // the heads: each cluster's representative and its next k + 10 members
  // (a representative is its own cluster's nearest member, so it comes
  // first unless an identical structure ties with it)
  std::vector<int64_t> hpos;
  std::vector<int> rep_slot(R, -1);
  for (int r = 0; r < R; ++r) {
    const int64_t rp = pos_of[rep[r]];
    if (cl[rep[r]] == r) {
      rep_slot[r] = (int)hpos.size();
      hpos.push_back(rp);
    }
    const int64_t m = std::min<int64_t>(first[r + 1] - first[r], (int64_t)k + 10);
    for (int64_t u = first[r]; u < first[r] + m; ++u)
      if (u != rp) hpos.push_back(u);
  }
  for (int r = 0; r < R; ++r)
    if (rep_slot[r] < 0) {  // a representative joined to another (identical) one
      rep_slot[r] = (int)hpos.size();
      hpos.push_back(pos_of[rep[r]]);
    }
  const int H = (int)hpos.size();
  ix.nhead = H;
  // library index of each position; the heads' digit rows
  std::vector<int> perm32(n);
  for (int64_t u = 0; u < n; ++u) perm32[u] = (int)ord[u];
  const int64_t hblocks = blocks_for(H);
  ix.rows = hblocks * kBlockRows;
  DevBuf dpos;
  bool ok = cudaMalloc(&ix.perm.p, (size_t)n * 4) == cudaSuccess &&
            cudaMalloc(&ix.info.p, (size_t)hblocks * kBlockStructs * 16) == cudaSuccess &&
            cudaMalloc(&ix.tinfo.p, (size_t)hblocks * kBlockStructs * 8) == cudaSuccess &&
            cudaMalloc(&ix.rep_slot.p, (size_t)R * 4) == cudaSuccess && cudaMalloc(&dpos.p, (size_t)H * 8) == cudaSuccess;
  for (int d = 0; d < 4 && ok; ++d) ok = cudaMalloc(&ix.dig[d].p, (size_t)ix.rows * bk.pitch * 2) == cudaSuccess;
  if (ok) {
    DigitPtrs dp{};
    for (int d = 0; d < 4; ++d) {
      dp.src[d] = static_cast<const __nv_bfloat16 *>(bk.dig[d].p);
      dp.dst[d] = static_cast<__nv_bfloat16 *>(ix.dig[d].p);
      ok = ok && cudaMemset(ix.dig[d].p, 0, (size_t)ix.rows * bk.pitch * 2) == cudaSuccess;
    }
    ok = ok && cudaMemset(ix.info.p, 0, (size_t)hblocks * kBlockStructs * 16) == cudaSuccess &&
         cudaMemset(ix.tinfo.p, 0, (size_t)hblocks * kBlockStructs * 8) == cudaSuccess &&
         cudaMemcpy(ix.perm.p, perm32.data(), (size_t)n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(ix.rep_slot.p, rep_slot.data(), (size_t)R * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(dpos.p, hpos.data(), (size_t)H * 8, cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
      k_gather_reps<<<H, 128>>>(dp, bk.pitch, static_cast<const int64_t *>(dpos.p), H,
                                static_cast<const SInfo *>(bk.info.p), static_cast<SInfo *>(ix.info.p),
                                static_cast<const float2 *>(bk.tinfo.p), static_cast<float2 *>(ix.tinfo.p));
      ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
    }
  }
  if (dpos.p) cudaFree(dpos.p);
  if (!ok) {
    cudaGetLastError();
    s->err = "library index: device memory";
    return BS_ERR_OOM;
  }
  bk.indexed = true;
  return BS_OK;
}

// After the slot's event: results to the requests (lock held; released
// while a clustering job's triangle is copied out of the slot).
void finish_slot(bs_server *s, Slot &sl, std::unique_lock<std::mutex> &lk) {
  const DevScalars &sc = *static_cast<const DevScalars *>(sl.hsc.p);
  if (sl.kind == 1) {
    Request *r = sl.reqs[0];
    std::string msg;
    bs_status st = BS_OK;
    if (sl.njobs == 1) st = collect_errors(sc, static_cast<const Job *>(sl.hback.p), 1, msg);
    else if (sc.err & kErrNonFinite) st = BS_ERR_NONFINITE, msg = "input coordinates contain NaN or Inf";
    if (st) {
      complete(s, r, st, msg);
    } else {
      const size_t tri = (size_t)(r->q * (r->q - 1) / 2);
      lk.unlock();  // the slot stays busy until the copy is done
      r->tri.assign(static_cast<const float *>(sl.htri.p), static_cast<const float *>(sl.htri.p) + tri);
      lk.lock();
      s->cluster_post.push_back(r);
      s->cv_clus.notify_one();
    }
  } else {
    const Bucket &bk = s->buckets[sl.bucket];
    const int k = s->top_k;
    const Job *back = static_cast<const Job *>(sl.hback.p);
    const int *hcn = sl.screen ? static_cast<const int *>(sl.hcand_n.p) : nullptr;
    std::vector<int> redo;
    // rows of query t of a request at row0 + t, or where an indexed screen
    // put it (mapped)
    auto take = [&](Request *r, int64_t row0, bool mapped) {
      const int64_t *hi = static_cast<const int64_t *>(sl.htopi.p);
      const float *hv = static_cast<const float *>(sl.htopv.p);
      r->idx.resize(r->q * k);
      r->val.resize(r->q * k);
      for (int64_t t = 0; t < r->q; ++t) {
        const int64_t src = mapped ? sl.row_of[row0 + t] : row0 + t;
        for (int e = 0; e < k; ++e) {
          r->idx[t * k + e] = hi[src * k + e];
          r->val[t * k + e] = (double)hv[src * k + e];
        }
      }
      r->pairs = r->q * bk.n;
    };
    const bool mapped_rows = !sl.row_of.empty();
    for (int j = 0; j < (int)sl.reqs.size(); ++j) {
      Request *r = sl.reqs[j];
      bs_status st = BS_OK;
      std::string msg;
      bool fell_back = false;
      if (s->precision == BS_PRECISION_MIXED) {
        st = collect_errors(sc, back + j, 1, msg);
        if (st == BS_ERR_UNSUPPORTED) {  // outside the bucket's grid: plain FP64 path
          fell_back = true;
          st = plain_fallback(s, sl, j);
          if (st == BS_OK) ++s->fallbacks;
          else msg = "plain fallback failed";
        } else if (st == BS_OK && hcn) {
          bool overflow = false;
          for (int64_t t = 0; t < r->q; ++t) overflow |= hcn[sl.row0[j] + t] > kCandCap;
          if (overflow) {  // more screen candidates than kept: certify the whole row
            redo.push_back(j);
            continue;
          }
        }
      } else if (sc.err & kErrNonFinite) {
        st = BS_ERR_NONFINITE;
        msg = "input coordinates contain NaN or Inf";
      }
      if (st == BS_OK) take(r, sl.row0[j], mapped_rows && !fell_back);
      complete(s, r, st, msg);
    }
    // rows whose screen band held more candidates than kept: every pair of
    // the request certified densely, synchronously on this slot -- without
    // the server lock (the slot stays busy, so nothing else uses its buffers),
    // so that the scheduler and the other slots' workers keep going
    std::vector<Request *> all = sl.reqs;
    for (int j : redo) {
      Request *r = all[j];
      sl.reqs.assign(1, r);
      lk.unlock();
      bs_status st = launch_query_batch(s, sl, false);
      if (st == BS_OK && cudaStreamSynchronize(sl.st) != cudaSuccess) st = BS_ERR_CUDA;
      std::string msg;
      if (st == BS_OK)
        st = collect_errors(*static_cast<const DevScalars *>(sl.hsc.p), static_cast<const Job *>(sl.hback.p), 1, msg);
      if (st == BS_OK) take(r, 0, false);
      lk.lock();
      complete(s, r, st, msg);
    }
  }
  sl.reqs.clear();
  sl.busy = false;
}

void cluster_loop(bs_server *s) {
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    s->cv_clus.wait(lk, [&] { return s->stop || !s->cluster_post.empty(); });
    if (s->cluster_post.empty()) {
      if (s->stop) break;
      continue;
    }
    Request *r = s->cluster_post.front();
    s->cluster_post.pop_front();
    lk.unlock();
    std::vector<int64_t> order(r->q), cl(r->q);
    std::vector<double> reach(r->q);
    const bs_status st = bs_optics(r->tri.data(), r->q, BS_OUT_F32, r->eps, r->min_points, order.data(), reach.data(),
                                   cl.data());
    r->tri.clear();
    r->tri.shrink_to_fit();
    lk.lock();
    r->labels = std::move(cl);
    r->pairs = r->q * (r->q - 1) / 2;
    complete(s, r, st, st ? "OPTICS failed" : "");
  }
}

void fail_batch(bs_server *s, Slot &sl, bs_status st, const std::string &msg) {
  for (Request *r : sl.reqs) complete(s, r, st, msg);
  sl.reqs.clear();
  sl.busy = false;
}

// A slot's worker: launches the batch the scheduler handed it (without the
// lock: an indexed screen waits for its pre-screen), waits for it, and
// completes its requests (with the lock).  Workers run side by side, so the
// host work of one batch overlaps the device work and host work of others.
void worker_loop(bs_server *s, Slot *slp) {
  cudaSetDevice(s->device);
  Slot &sl = *slp;
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    sl.cv.wait(lk, [&] { return sl.has_work || sl.quit; });
    if (!sl.has_work) break;
    sl.has_work = false;
    const int kind = sl.kind;
    const int64_t rows = kind == 0 ? [&] {
      int64_t t = 0;
      for (const Request *r : sl.reqs) t += r->q;
      return t;
    }() : sl.reqs[0]->q;
    const int nreq = (int)sl.reqs.size(), bucket = sl.bucket;
    lk.unlock();
    t_grow_dev = t_grow_host = 0;
    t_grow_ms = 0.0;
    const Clock::time_point t_lb = Clock::now();
    bs_status st = kind == 0 ? launch_query_batch(s, sl, true) : launch_cluster_batch(s, sl);
    const Clock::time_point t_le = Clock::now();
    cudaError_t e = cudaSuccess;
    if (st == BS_OK) e = cudaEventSynchronize(sl.ev);
    const Clock::time_point t_ev = Clock::now();
    lk.lock();
    if (st) {
      cudaGetLastError();
      cudaStreamSynchronize(sl.st);
      fail_batch(s, sl, st, st == BS_ERR_OOM ? "device memory" : "batch launch failed");
    } else if (e != cudaSuccess) {
      cudaGetLastError();
      fail_batch(s, sl, BS_ERR_CUDA, cudaGetErrorString(e));
    } else {
      finish_slot(s, sl, lk);
    }
    if (!s->trace_path.empty()) {
      char line[256];
      snprintf(line, sizeof line, "B,%d,%lld,%d,%d,%lld,%d,%.3f,%.3f,%.3f,%.3f,%.3f,%d,%d,%.3f",
               [&] {
                 for (size_t i = 0; i < s->slots.size(); ++i)
                   if (s->slots[i].get() == slp) return (int)i;
                 return -1;
               }(),
               (long long)sl.batch_id, kind, bucket, (long long)rows, nreq, ms_between(s->t0, sl.t_hand),
               ms_between(s->t0, t_lb), ms_between(s->t0, t_le), ms_between(s->t0, t_ev),
               ms_between(s->t0, Clock::now()), t_grow_dev, t_grow_host, t_grow_ms);
      s->trace.emplace_back(line);
    }
    s->cv_work.notify_one();  // the slot is free again
  }
}

// The scheduler: forms batches from the queue and hands them to idle slots.
void sched_loop(bs_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    bool progress = false;
    for (auto &up : s->slots) {
      Slot &sl = *up;
      if (sl.busy || s->queue.empty()) continue;
      // form a batch: the oldest request, plus same-bucket queries behind it
      std::vector<Request *> batch{s->queue.front()};
      const Request *r0 = batch[0];
      int64_t rows = r0->q;
      if (r0->kind == 0) {
        for (size_t i = 1; i < s->queue.size(); ++i) {
          Request *r = s->queue[i];
          if (r->kind != 0 || r->bucket != r0->bucket || rows + r->q > s->max_rows) continue;
          batch.push_back(r);
          rows += r->q;
        }
      }
      // admission by device memory: shrink the batch until it fits the
      // budget left by the other slots (idle slots give theirs back first)
      size_t need = batch_bytes(s, batch);
      if (s->used - slot_bytes(sl) + need * 5 / 4 > s->budget) {
        for (auto &o : s->slots)
          if (!o->busy && o.get() != &sl) slot_release(s, *o);
      }
      while (batch.size() > 1 && s->used - slot_bytes(sl) + need * 5 / 4 > s->budget) {
        batch.pop_back();
        need = batch_bytes(s, batch);
      }
      if (s->used - slot_bytes(sl) + need * 5 / 4 > s->budget) {
        bool others = false;
        for (auto &o : s->slots) others |= o->busy;
        if (others) break;  // wait for memory to free up
        Request *r = s->queue.front();
        s->queue.pop_front();
        complete(s, r, BS_ERR_BUDGET, "request larger than the server's device memory budget");
        progress = true;
        continue;
      }
      for (Request *r : batch) {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
        r->batch = s->batch_seq;
      }
      sl.batch_id = s->batch_seq++;
      sl.t_hand = Clock::now();
      sl.busy = true;
      sl.reqs = batch;
      sl.kind = r0->kind;
      sl.bucket = r0->bucket;
      ++s->batches;
      if (r0->kind == 0) s->rows_batched += rows;
      sl.has_work = true;
      sl.cv.notify_one();
      progress = true;
    }
    if (s->stop && s->queue.empty()) {
      bool busy = false;
      for (auto &up : s->slots) busy |= up->busy;
      if (!busy) break;
    }
    if (!progress) s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
  }
  for (auto &up : s->slots) up->quit = true;
  for (auto &up : s->slots) up->cv.notify_one();
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  const size_t k = std::min(v.size() - 1, (size_t)std::floor(p * (double)(v.size() - 1) + 0.5));
  std::nth_element(v.begin(), v.begin() + k, v.end());
  return v[k];
}

}  // namespace
}  // namespace bs

using namespace bs;

extern "C" {

BS_API const char *bs_server_last_error(const bs_server *s) { return s ? s->err.c_str() : "null server"; }

BS_API bs_status bs_server_create(bs_server **out, int32_t device, const bs_server_config *cfg) {
  if (!out || !cfg) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->nbuckets < 1 || !cfg->bucket_L || !cfg->bucket_n || !cfg->bucket_xyz) return BS_ERR_INVALID_ARG;
  if (cfg->top_k < 1 || cfg->top_k > kTopkMax) return BS_ERR_INVALID_ARG;
  if (cfg->precision != BS_PRECISION_MIXED && cfg->precision != BS_PRECISION_PLAIN64) return BS_ERR_INVALID_ARG;
  for (int b = 0; b < cfg->nbuckets; ++b) {
    if (cfg->bucket_L[b] < 1 || cfg->bucket_n[b] < 1 || !cfg->bucket_xyz[b]) return BS_ERR_INVALID_ARG;
    for (int c = 0; c < b; ++c)
      if (cfg->bucket_L[c] == cfg->bucket_L[b]) return BS_ERR_INVALID_ARG;  // one bucket per length
    if (cfg->bucket_n[b] >= kMaxGlobalStructs) return BS_ERR_UNSUPPORTED;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return BS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return BS_ERR_INVALID_ARG;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || !(prop.major == 10 && prop.minor == 3))
    return BS_ERR_NO_DEVICE;
  bs_server *s = new (std::nothrow) bs_server();
  if (!s) return BS_ERR_OOM;
  s->device = device;
  s->num_sms = prop.multiProcessorCount;
  s->top_k = cfg->top_k;
  s->max_inflight = cfg->max_inflight > 0 ? cfg->max_inflight : 4;
  s->max_rows = cfg->max_batch_rows > 0 ? cfg->max_batch_rows : 4096;
  s->precision = cfg->precision;
  s->tol = (float)(cfg->tolerance > 0 ? cfg->tolerance : 1e-4);
  if (const char *tp = getenv("BS_SERVER_TRACE")) s->trace_path = tp;
  cudaSetDevice(device);
  if (mixed_tc_prepare() != cudaSuccess || screen_tc_prepare() != cudaSuccess || prep_prepare() != cudaSuccess ||
      !get_encoder(&s->encode).empty()) {
    delete s;
    return BS_ERR_CUDA;
  }
  {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next batch
    if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      cudaGetLastError();
      bs_server_destroy(s);
      return BS_ERR_CUDA;
    }
  }
  s->buckets.resize(cfg->nbuckets);
  for (int b = 0; b < cfg->nbuckets; ++b) {
    s->buckets[b].L = cfg->bucket_L[b];
    s->buckets[b].n = cfg->bucket_n[b];
    const bs_status st = build_bucket(s, s->buckets[b], cfg->bucket_xyz[b]);
    if (st) {
      const std::string e = s->err;
      bs_server_destroy(s);
      return st;
    }
  }
  for (int i = 0; i < s->max_inflight; ++i) {
    auto sl = std::make_unique<Slot>();
    int lo_pri = 0, hi_pri = 0;
    cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri);
    if (cudaStreamCreateWithFlags(&sl->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming | cudaEventBlockingSync) != cudaSuccess ||
        cudaStreamCreateWithPriority(&sl->pst, cudaStreamNonBlocking, hi_pri) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl->pev, cudaEventDisableTiming) != cudaSuccess) {
      bs_server_destroy(s);
      return BS_ERR_CUDA;
    }
    s->slots.push_back(std::move(sl));
  }
  // library indexes of the large buckets (mixed precision: they prune screens)
  const int64_t index_min = cfg->index_min > 0 ? cfg->index_min : (cfg->index_min < 0 ? INT64_MAX : kIndexMinDefault);
  for (int b = 0; b < cfg->nbuckets && s->precision == BS_PRECISION_MIXED; ++b) {
    if (cfg->bucket_n[b] < index_min || cfg->bucket_n[b] < 2) continue;
    const size_t bytes = (size_t)cfg->bucket_n[b] * cfg->bucket_L[b] * 3 * 8;
    std::vector<double> hx;
    const double *src = cfg->bucket_xyz[b];
    if (is_device_ptr(src)) {
      hx.resize(bytes / 8);
      if (cudaMemcpy(hx.data(), src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
        bs_server_destroy(s);
        return BS_ERR_CUDA;
      }
      src = hx.data();
    }
    const bs_status st = build_index(s, b, src);
    if (st) {
      bs_server_destroy(s);
      return st;
    }
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  s->budget = cfg->hbm_budget ? cfg->hbm_budget : free_b / 2;
  if (const bs_status st = reserve_slots(s, cfg)) {
    bs_server_destroy(s);
    return st;
  }
  s->t0 = Clock::now();
  for (auto &up : s->slots) up->worker = std::thread(worker_loop, s, up.get());
  s->sched = std::thread(sched_loop, s);
  s->clus = std::thread(cluster_loop, s);
  *out = s;
  return BS_OK;
}

BS_API void bs_server_destroy(bs_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_clus.notify_all();
  if (s->sched.joinable()) s->sched.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto &up : s->slots) up->quit = true;
  }
  for (auto &up : s->slots) {
    up->cv.notify_one();
    if (up->worker.joinable()) up->worker.join();
  }
  if (s->clus.joinable()) s->clus.join();
  cudaSetDevice(s->device);
  for (auto &up : s->slots) {
    Slot &sl = *up;
    if (sl.pst) cudaStreamSynchronize(sl.pst);
    if (sl.st) {
      cudaStreamSynchronize(sl.st);
      slot_release(s, sl);
    }
    each_host(sl, [](HostBuf &h) {
      if (h.p) cudaFreeHost(h.p);
    });
    for (void *p : sl.retired) cudaFreeHost(p);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.st) cudaStreamDestroy(sl.st);
    if (sl.pev) cudaEventDestroy(sl.pev);
    if (sl.pst) {
      cudaStreamSynchronize(sl.pst);
      cudaStreamDestroy(sl.pst);
    }
  }
  if (s->pool) cudaMemPoolDestroy(s->pool);
  for (Bucket &bk : s->buckets) free_bucket(bk);
  for (auto &kv : s->reqs) delete kv.second;
  if (!s->trace_path.empty()) {
    if (FILE *f = fopen(s->trace_path.c_str(), "a")) {  // servers of one process append
      fprintf(f, "# server\n# B,slot,batch,kind,bucket,rows,nreq,hand_ms,launch_begin_ms,launch_end_ms,event_ms,finish_ms,"
                 "dev_grows,host_grows,grow_ms\n# R,id,kind,bucket,q,submit_ms,done_ms,batch,status\n");
      for (const std::string &l : s->trace) fprintf(f, "%s\n", l.c_str());
      fclose(f);
    }
  }
  delete s;
}

static bs_status submit_common(bs_server *s, Request *r, int64_t *ticket) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete r;
    return BS_ERR_INVALID_ARG;
  }
  r->id = s->next_id++;
  r->t_submit = Clock::now();
  s->reqs[r->id] = r;
  s->queue.push_back(r);
  *ticket = r->id;
  s->cv_work.notify_one();
  return BS_OK;
}

BS_API bs_status bs_server_submit(bs_server *s, const double *xyz, int32_t q, int32_t L, int64_t *ticket) {
  if (!s || !xyz || !ticket || q < 1) return BS_ERR_INVALID_ARG;
  int bucket = -1;
  for (int b = 0; b < (int)s->buckets.size(); ++b)
    if (s->buckets[b].L == L) bucket = b;
  if (bucket < 0) return BS_ERR_INVALID_ARG;
  Request *r = new (std::nothrow) Request();
  if (!r) return BS_ERR_OOM;
  r->kind = 0;
  r->bucket = bucket;
  r->L = L;
  r->q = q;
  r->xyz.assign(xyz, xyz + (size_t)q * L * 3);
  return submit_common(s, r, ticket);
}

BS_API bs_status bs_server_submit_cluster(bs_server *s, const double *xyz, int64_t n, int32_t L, double eps,
                                          int32_t min_points, int64_t *ticket) {
  if (!s || !xyz || !ticket || n < 2 || L < 1 || !(eps > 0) || min_points < 1) return BS_ERR_INVALID_ARG;
  Request *r = new (std::nothrow) Request();
  if (!r) return BS_ERR_OOM;
  r->kind = 1;
  r->L = L;
  r->q = n;
  r->eps = eps;
  r->min_points = min_points;
  r->xyz.assign(xyz, xyz + (size_t)n * L * 3);
  return submit_common(s, r, ticket);
}

BS_API bs_status bs_server_poll(bs_server *s, int64_t ticket, int32_t *done) {
  if (!s || !done) return BS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return BS_ERR_INVALID_ARG;
  *done = it->second->done ? 1 : 0;
  return BS_OK;
}

static bs_status wait_common(bs_server *s, int64_t ticket, double timeout_s, int kind, Request **out) {
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second->kind != kind) return BS_ERR_INVALID_ARG;
  Request *r = it->second;
  auto pred = [&] { return r->done; };
  if (timeout_s > 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return BS_ERR_TIMEOUT;
  } else {
    s->cv_done.wait(lk, pred);
  }
  s->reqs.erase(it);
  *out = r;
  if (r->status) s->err = r->err;
  return r->status;
}

BS_API bs_status bs_server_wait(bs_server *s, int64_t ticket, int64_t *hit_index, double *hit_rmsd, double timeout_s) {
  if (!s || !hit_index || !hit_rmsd) return BS_ERR_INVALID_ARG;
  Request *r = nullptr;
  const bs_status st = wait_common(s, ticket, timeout_s, 0, &r);
  if (r) {
    if (st == BS_OK) {
      memcpy(hit_index, r->idx.data(), r->idx.size() * 8);
      memcpy(hit_rmsd, r->val.data(), r->val.size() * 8);
    }
    delete r;
  }
  return st;
}

BS_API bs_status bs_server_wait_cluster(bs_server *s, int64_t ticket, int64_t *cluster_of, double timeout_s) {
  if (!s || !cluster_of) return BS_ERR_INVALID_ARG;
  Request *r = nullptr;
  const bs_status st = wait_common(s, ticket, timeout_s, 1, &r);
  if (r) {
    if (st == BS_OK) memcpy(cluster_of, r->labels.data(), r->labels.size() * 8);
    delete r;
  }
  return st;
}

BS_API bs_status bs_server_cancel(bs_server *s, int64_t ticket, int32_t *cancelled) {
  if (!s || !cancelled) return BS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return BS_ERR_INVALID_ARG;
  Request *r = it->second;
  auto q = std::find(s->queue.begin(), s->queue.end(), r);
  *cancelled = 0;
  if (q == s->queue.end() || r->done) return BS_OK;  // running or done: its wait returns its result
  s->queue.erase(q);
  complete(s, r, BS_ERR_CANCELLED, "cancelled before it ran");
  *cancelled = 1;
  return BS_OK;
}

BS_API bs_status bs_server_get_stats(bs_server *s, bs_server_stats *out) {
  if (!s || !out) return BS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = bs_server_stats{};
  out->queries_done = s->qdone;
  out->clusters_done = s->cdone;
  out->pairs = s->pairs;
  out->batches = s->batches;
  out->plain_fallbacks = s->fallbacks;
  int64_t pending = 0;
  for (auto &kv : s->reqs) pending += kv.second->done ? 0 : 1;
  out->pending = pending;
  out->p50_ms = percentile(s->lat, 0.50);
  out->p99_ms = percentile(s->lat, 0.99);
  out->max_ms = s->lat.empty() ? 0.0 : *std::max_element(s->lat.begin(), s->lat.end());
  double sum = 0.0;
  for (double v : s->lat) sum += v;
  out->mean_ms = s->lat.empty() ? 0.0 : sum / (double)s->lat.size();
  out->cluster_p50_ms = percentile(s->clat, 0.50);
  out->cluster_p99_ms = percentile(s->clat, 0.99);
  out->seconds = ms_between(s->t0, Clock::now()) * 1e-3;
  out->pairs_per_s = out->seconds > 0 ? (double)s->pairs / out->seconds : 0.0;
  out->mean_batch_rows = s->batches ? (double)s->rows_batched / (double)s->batches : 0.0;
  out->pairs_screened = s->screened;
  return BS_OK;
}

BS_API bs_status bs_server_reset_stats(bs_server *s) {
  if (!s) return BS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->lat.clear();
  s->clat.clear();
  s->qdone = s->cdone = s->pairs = s->batches = s->fallbacks = s->rows_batched = 0;
  s->screened = 0;
  if (!s->trace_path.empty()) s->trace.emplace_back("# reset");  // later times count from here
  s->t0 = Clock::now();
  return BS_OK;
}

}  // extern "C"
