// plan.cu -- the mixed-path launch plan (jobs, block map, tile table), the
// tensor maps, and the device call sequence shared by every entry point.
#include <stdio.h>

#include <algorithm>
#include <numeric>

#include "engine.h"

namespace bs {

std::string make_symmetric_plan(const std::vector<JobSpec> &specs, float tol, bool with_tiles, Plan &plan) {
  plan = Plan{};
  const int nj = (int)specs.size();
  if (nj > 65535) return "more than 65535 structure sets in one call";
  int64_t blk = 0;
  int pitch = kKChunk;
  plan.jobs.resize(nj);
  // structure blocks are laid out job by job in the order the tiles run
  // (longest chains first, so that long tiles do not trail the launch):
  // a band of consecutive tiles then covers a contiguous range of blocks
  std::vector<int> order(nj);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return specs[a].L > specs[b].L; });
  for (int j : order) {
    const JobSpec &s = specs[j];
    Job &jb = plan.jobs[j];
    jb = Job{};
    jb.xyz = s.xyz;
    jb.n = s.n;
    jb.first_a = blk * kBlockStructs;
    jb.first_b = jb.first_a;
    jb.n_b = s.n;
    jb.out = s.out;
    jb.L = s.L;
    jb.lp = lp_for(s.L);
    jb.mode = 0;
    jb.fixed_scale = 0;
    jb.scale_min = -1000;
    jb.tol = tol;
    jb.allow_long = 1;
    jb.narrow = s.narrow ? 1 : 0;
    const int64_t nb = blocks_for(s.n);
    for (int64_t b = 0; b < nb; ++b) plan.jobmap.push_back(j);
    blk += nb;
    pitch = std::max(pitch, pitch_for(s.L));
  }
  if (blk * kBlockStructs > kMaxGlobalStructs) return "more than 2^24 structures (padded to blocks of 40) in one call";
  if (pitch > prep_max_pitch()) {
    char buf[128];
    snprintf(buf, sizeof(buf), "chain length above the mixed path's limit of %d atoms", prep_max_pitch());
    return buf;
  }
  plan.nblocks = blk;
  plan.pitch = pitch;
  if (!with_tiles) return "";
  constexpr int64_t SA = 32, SB = 64;  // super-block: 32 A blocks x 64 B blocks
  // two passes over the same loops: the count (per A block and super-block),
  // then the tiles into a table of exactly that size
  for (int pass = 0; pass < 2; ++pass) {
    int64_t count = 0;
    for (int j : order) {
      const Job &jb = plan.jobs[j];
      if (jb.n < 2) continue;
      // B blocks of bs structures; tile (I, J) holds a pair i < j iff
      // bs J + bs - 1 > 40 I, i.e. J >= r I with r = 40 / bs
      const int64_t bs = jb.narrow ? kNarrowStructs : kBStructs, r = kBlockStructs / bs;
      const int64_t nba = blocks_for(jb.n), nbb = (jb.n + bs - 1) / bs;
      const int64_t a0 = jb.first_a / kBlockStructs, b0 = jb.first_a / bs;
      // a row range keeps the tiles of its A blocks (40-structure multiples)
      const int64_t ilo = specs[j].row_lo / kBlockStructs;
      const int64_t ihi = specs[j].row_hi < 0 ? nba : (specs[j].row_hi + kBlockStructs - 1) / kBlockStructs;
      for (int64_t sa = 0; sa < nba; sa += SA)
        for (int64_t sb = r * sa; sb < nbb; sb += SB * r / 2)
          for (int64_t I = std::max(sa, ilo); I < std::min(std::min(sa + SA, nba), ihi); ++I) {
            const int64_t jlo = std::max(sb, r * I), jhi = std::min(sb + SB * r / 2, nbb);
            if (pass == 0) {
              count += std::max<int64_t>(0, jhi - jlo);
              continue;
            }
            for (int64_t J = jlo; J < jhi; ++J) plan.tiles.push_back(Tile{(int)(a0 + I), (int)(b0 + J), j, 0});
          }
    }
    if (pass == 0) plan.tiles.reserve((size_t)count);
  }
  return "";
}

std::string get_encoder(PFN_cuTensorMapEncodeTiled_v12000 *out) {
  if (*out) return "";
  cudaDriverEntryPointQueryResult q;
  void *fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return "cuTensorMapEncodeTiled unavailable in the CUDA driver";
  }
  *out = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return "";
}

std::string encode_maps(PFN_cuTensorMapEncodeTiled_v12000 encode, const MixedBuffers &b, CUtensorMap tm[7]) {
  // maps 0-3: A operand boxes (64 atoms x 128 rows) of e0, e1, e2, d2/32;
  // maps 4-6: B boxes (64 x 64) of e0, e1, e2
  for (int m = 0; m < 7; ++m) {
    const bool a = m < 4;
    const void *base = a ? (const void *)b.dig_a[m] : (const void *)b.dig_b[m - 4];
    const int64_t pitch = a ? b.pitch_a : b.pitch_b, rows = a ? b.rows_a : b.rows_b;
    cuuint64_t gdim[2] = {(cuuint64_t)pitch, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)pitch * 2};
    cuuint32_t box[2] = {(cuuint32_t)kKChunk, a ? 128u : 64u};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&tm[m], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), gdim, gstride, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      char buf[96];
      snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d) for map %d", (int)r, m);
      return buf;
    }
  }
  return "";
}

void make_bands(const Plan &plan, int64_t n, int bands, Readback &rb) {
  constexpr int64_t SA = 32;  // A blocks per super-row (make_symmetric_plan)
  rb.tile_end.clear();
  rb.elem_end.clear();
  auto off = [n](int64_t r) { return r * n - r * (r + 1) / 2; };  // packed index of (r, r + 1)
  const int64_t total = n * (n - 1) / 2, want = std::max<int64_t>(1, total / std::max(1, bands));
  int64_t last = 0;
  const int64_t nt = (int64_t)plan.tiles.size();
  for (int64_t t = 1; t < nt; ++t) {
    const int64_t s = plan.tiles[t].a_blk / SA;
    if (s == plan.tiles[t - 1].a_blk / SA) continue;
    const int64_t e = off(std::min(n, s * SA * kBlockStructs));
    if (e >= total) break;  // the rest holds no pairs: it joins the last band
    // equal bands, then each half of what is left (down to a sixteenth of a
    // band): the copy of the last band, which nothing hides, stays short
    const int64_t rem = total - last;
    const int64_t target = rem > 2 * want ? want : std::max<int64_t>(rem / 2, std::max<int64_t>(1, want / 16));
    if (e - last >= target) {
      rb.tile_end.push_back(t);
      rb.elem_end.push_back(e);
      last = e;
    }
  }
  rb.tile_end.push_back(nt);
  rb.elem_end.push_back(total);
}

void make_set_bands(const Plan &plan, int bands, Readback &rb) {
  rb.tile_end.clear();
  rb.elem_end.clear();
  rb.copies.clear();
  const int64_t nt = (int64_t)plan.tiles.size();
  int64_t total = 0;
  for (const Job &jb : plan.jobs) total += jb.n * (jb.n - 1) / 2;
  const int64_t want = std::max<int64_t>(1, total / std::max(1, bands));
  int64_t done = 0, band = 0;
  for (int64_t t = 0; t < nt; ++t) {
    if (t + 1 < nt && plan.tiles[t + 1].job == plan.tiles[t].job) continue;
    const Job &jb = plan.jobs[plan.tiles[t].job];  // the last tile of a job
    band += jb.n * (jb.n - 1) / 2;
    const int64_t rem = total - done;
    const int64_t target = rem > 2 * want ? want : std::max<int64_t>(rem / 2, std::max<int64_t>(1, want / 16));
    if (band >= target || t + 1 == nt) {
      rb.tile_end.push_back(t + 1);
      done += band;
      band = 0;
    }
  }
  if (rb.tile_end.empty()) rb.tile_end.push_back(nt);
  rb.copies.resize(rb.tile_end.size());
}

cudaError_t enqueue_mixed(const Plan &plan, const MixedBuffers &b, const Job *job_stage, const CUtensorMap tm[7],
                          int num_sms, cudaStream_t st, cudaEvent_t *ev, bool capturing, float *dbg,
                          const Readback *rb) {
  auto rec = [&](int k) -> cudaError_t {
    if (!ev) return cudaSuccess;
    return cudaEventRecordWithFlags(ev[k], st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
  };
  const int nj = (int)plan.jobs.size();
  cudaError_t e;
  if ((e = rec(0)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(b.jobs, job_stage, (size_t)nj * sizeof(Job), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(b.sc, 0, sizeof(DevScalars), st)) != cudaSuccess) return e;
  // banded preparation: every band's uploads are queued now on their own
  // stream; each band is prepared once its uploads have landed
  const bool band_prep = rb && !rb->struct_end.empty();
  if (band_prep) {
    for (size_t k = 0; k < rb->tile_end.size(); ++k) {
      for (const Readback::Upload &u : rb->uploads[k])
        if (u.bytes && (e = cudaMemcpyAsync(u.dev, u.host, u.bytes, cudaMemcpyHostToDevice, rb->upload)) !=
                           cudaSuccess)
          return e;
      if ((e = cudaEventRecord(rb->up_ev[k], rb->upload)) != cudaSuccess) return e;
    }
  }
  PrepArgs p{};
  p.jobs = b.jobs;
  p.njobs = nj;
  p.job_of_struct_block = b.jobmap;
  p.nblocks = plan.nblocks;
  p.ctr = b.ctr;
  for (int d = 0; d < 4; ++d) p.dig[d] = b.dig_a[d];
  p.pitch = b.pitch_a;
  p.info = b.info_a;
  p.tinfo = b.tinfo_a;
  p.sc = b.sc;
  if (!band_prep) {
    if ((e = launch_prep_mixed(p, st)) != cudaSuccess) return e;
    if ((e = rec(1)) != cudaSuccess) return e;
  }
  if (!plan.tiles.empty()) {
    // strip records carry their shape; tiles get theirs from the prepared jobs
    if (!plan.strips && !band_prep &&
        (e = launch_tile_shapes(b.tiles, (int64_t)plan.tiles.size(), b.jobs, num_sms, st)) != cudaSuccess)
      return e;
    TcArgs a{};
    a.tiles = b.tiles;
    a.ntiles = (int64_t)plan.tiles.size();
    a.jobs = b.jobs;
    a.info_a = b.info_a;
    a.info_b = b.info_b;
    a.tinfo_a = b.tinfo_a;
    a.tinfo_b = b.tinfo_b;
    a.sc = b.sc;
    a.flags = b.flags;
    a.flag_cap = b.flag_cap;
    a.dbg = dbg;
    a.num_sms = num_sms;
    a.wait_ns = b.wait_ns;
    // launches of screen jobs only run the screen-shaped kernel
    bool all_screen = nj > 0;
    for (const Job &jb : plan.jobs) all_screen = all_screen && jb.screen;
    RefineArgs r{};
    r.da = DigitsView{b.dig_a[0], b.dig_a[1], b.dig_a[2], b.pitch_a};
    r.db = DigitsView{b.dig_b[0], b.dig_b[1], b.dig_b[2], b.pitch_b};
    r.info_a = b.info_a;
    r.info_b = b.info_b;
    r.jobs = b.jobs;
    r.njobs = nj;
    r.sc = b.sc;
    r.flags = b.flags;
    r.cap = b.flag_cap;
    r.num_sms = num_sms;
    if (!rb) {
      if ((e = all_screen ? launch_screen_tc(tm, a, plan.strips, st) : launch_mixed_tc(tm, a, st)) != cudaSuccess)
        return e;
      if ((e = rec(2)) != cudaSuccess) return e;
      // screen tiles flag no pair: nothing to recompute
      r.scan_lo = plan.scan_lo;
      r.scan_hi = plan.scan_hi;
      if (!all_screen && (e = launch_refine(r, st)) != cudaSuccess) return e;
    } else {
      const size_t nb = rb->tile_end.size();
      const bool sets = !rb->copies.empty();
      r.mark = true;
      for (size_t k = 0; k < nb; ++k) {
        const int64_t t0 = k ? rb->tile_end[k - 1] : 0, e0 = sets ? 0 : (k ? rb->elem_end[k - 1] : 0);
        a.tiles = b.tiles + t0;
        a.ntiles = rb->tile_end[k] - t0;
        if (band_prep) {
          // this band's structures, once uploaded, and its tiles' shapes
          if ((e = cudaStreamWaitEvent(st, rb->up_ev[k], 0)) != cudaSuccess) return e;
          p.s_lo = k ? rb->struct_end[k - 1] : 0;
          p.s_hi = rb->struct_end[k];
          if ((e = launch_prep_mixed(p, st)) != cudaSuccess) return e;
          if (k == 0 && (e = rec(1)) != cudaSuccess) return e;
          if (a.ntiles > 0 && (e = launch_tile_shapes(b.tiles + t0, a.ntiles, b.jobs, num_sms, st)) != cudaSuccess)
            return e;
        }
        // each launch hands out its tiles from a counter at zero
        if (k > 0 && (e = cudaMemsetAsync(&b.sc->tile_next, 0, sizeof(unsigned long long), st)) != cudaSuccess)
          return e;
        if (a.ntiles > 0 && (e = launch_mixed_tc(tm, a, st)) != cudaSuccess) return e;
        if (k + 1 == nb && (e = rec(2)) != cudaSuccess) return e;
        r.scan_lo = sets ? 0 : e0;
        r.scan_hi = sets ? -1 : rb->elem_end[k];
        if ((e = launch_refine(r, st)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(rb->ev[k], st)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(rb->copy, rb->ev[k], 0)) != cudaSuccess) return e;
        if (sets) {
          for (const Readback::Copy &c : rb->copies[k])
            if (c.bytes && (e = cudaMemcpyAsync(c.host, c.dev, c.bytes, cudaMemcpyDeviceToHost, rb->copy)) !=
                               cudaSuccess)
              return e;
          continue;
        }
        const size_t bytes = (size_t)(rb->elem_end[k] - e0) * rb->esz;
        if (bytes && (e = cudaMemcpyAsync(rb->host + (size_t)e0 * rb->esz, rb->dev + (size_t)e0 * rb->esz, bytes,
                                          cudaMemcpyDeviceToHost, rb->copy)) != cudaSuccess)
          return e;
      }
      if ((e = cudaEventRecord(rb->ev[nb], rb->copy)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(st, rb->ev[nb], 0)) != cudaSuccess) return e;
    }
  } else {
    if ((e = rec(2)) != cudaSuccess) return e;
  }
  return rec(3);
}

bs_status collect_errors(const DevScalars &sc, const Job *jobs, int njobs, std::string &msg) {
  char buf[256];
  if (sc.err & kErrTimeout) {
    msg = "a device-side wait timed out";
    return BS_ERR_TIMEOUT;
  }
  if (sc.err & kErrInternal) {
    msg = "device-side invariant violated";
    return BS_ERR_INTERNAL;
  }
  for (int j = 0; j < njobs; ++j) {
    if (jobs[j].err & kErrNonFinite) {
      snprintf(buf, sizeof(buf), "structure set %d: input coordinates contain NaN or Inf", j);
      msg = buf;
      return BS_ERR_NONFINITE;
    }
  }
  for (int j = 0; j < njobs; ++j) {
    if (jobs[j].err & kErrUnsupported) {
      snprintf(buf, sizeof(buf),
               "structure set %d: coordinates beyond +-32768 A, or no coordinate grid meets the exactness bound "
               "(chain of %d atoms)",
               j, jobs[j].L);
      msg = buf;
      return BS_ERR_UNSUPPORTED;
    }
  }
  return BS_OK;
}

}  // namespace bs
