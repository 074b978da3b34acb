// batch_host.cu — resident volume slots and batched rendering: a fixed list
// of frames over the resident volumes, one persistent launch per method,
// captured with the resets of its counters in one CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "ctx.cuh"

using namespace cvr::ctxutil;

struct cvr_batch {
  cvr_ctx* ctx = nullptr;
  int n_jobs = 0;
  BatchExtJob* d_ext = nullptr;
  int n_ext = 0;
  unsigned ext_blocks = 0;
  int ext_max_table = 0;
  int ext_variant = 0;
  int ext_threads = 128;
  float4* d_tables = nullptr;
  int n_sur = 0;
  bool sur_tex = false;
  unsigned int* d_counters = nullptr;  // [0] extinction tiles, [1 + k] surrogate rays of launch k
  unsigned long long* d_stats = nullptr;  // 3 per job, in the caller's job order
  bool ext_compact = false;
  bool ext_aligned = false;  // every job: an aligned shadow table and aligned AO boxes (or AO off)
  std::vector<uint4*> sat32;              // the batch's own compact SATs, one per volume slot used
  std::vector<uint4*> walks;              // their walk tables, one per (slot, walk axis, depth) in use
  std::vector<long long> walk_keys;
  cudaGraphExec_t graph = nullptr;
  ~cvr_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    void* bufs[] = {d_ext, d_tables, d_counters, d_stats};
    for (void* p : bufs)
      if (p) cudaFree(p);
    for (uint4* p : sat32)
      if (p) cudaFree(p);
    for (uint4* p : walks)
      if (p) cudaFree(p);
  }
};

namespace {

// Makes slot s current; returns the slot that was.
int select_slot(cvr_ctx* c, int s) {
  int prev = c->cur_slot;
  if (s != prev) {
    swap_volume(c, c->slots[prev]);
    swap_volume(c, c->slots[s]);
    c->cur_slot = s;
  }
  return prev;
}

// Dominant axis of a job's directional light (the walk axis of its shadow
// table), 3 for other lights: jobs that share a volume and this axis read
// the same walk table.
int job_walk_axis(const cvr_job& j) {
  if (j.light.type != CVR_LIGHT_DIRECTIONAL) return 3;
  const float a[3] = {std::fabs(j.light.forward[0]), std::fabs(j.light.forward[1]), std::fabs(j.light.forward[2])};
  return (a[2] > a[0] && a[2] > a[1]) ? 2 : (a[1] > a[0] ? 1 : 0);
}

double job_cost(const cvr_job& j, const cvr_ctx* c) {
  const VolSlot& v = c->slots[j.volume];
  int nx = j.volume == c->cur_slot ? c->nx : v.nx, ny = j.volume == c->cur_slot ? c->ny : v.ny,
      nz = j.volume == c->cur_slot ? c->nz : v.nz;
  return (double)j.width * j.height * std::sqrt((double)nx * nx + (double)ny * ny + (double)nz * nz);
}

}  // namespace

extern "C" {

cvr_status cvr_select_volume(cvr_ctx* c, int slot) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (slot < 0 || slot >= CVR_MAX_VOLUMES) return fail(c, CVR_ERR_INVALID_ARG, "cvr_select_volume: slot out of range");
  select_slot(c, slot);
  return CVR_OK;
}

int cvr_current_volume(cvr_ctx* c) { return c ? c->cur_slot : -1; }

cvr_status cvr_batch_create(cvr_ctx* c, const cvr_job* jobs, int n_jobs, cvr_batch** out) {
  if (!c || !jobs || n_jobs <= 0 || !out) return fail(c, CVR_ERR_INVALID_ARG, "cvr_batch_create: bad arguments");
  *out = nullptr;
  for (int i = 0; i < n_jobs; ++i) {
    const cvr_job& j = jobs[i];
    if (j.volume < 0 || j.volume >= CVR_MAX_VOLUMES || !j.params)
      return fail(c, CVR_ERR_INVALID_ARG, "cvr_batch_create: bad job (volume slot or params)");
    if (j.method == CVR_METHOD_EXTINCTION ? j.params_size != sizeof(cvr_ext_params)
                                          : (j.method == CVR_METHOD_SURROGATE ? j.params_size != sizeof(cvr_gt_params)
                                                                              : true))
      return fail(c, CVR_ERR_INVALID_ARG, "cvr_batch_create: jobs must be extinction or surrogate with their params");
  }
  if (c->lc_dims[0] > 0)
    return fail(c, CVR_ERR_UNSUPPORTED, "cvr_batch_create: the light cache is per frame, not batched (turn it off)");
  if (c->ms_mode != CVR_MULTISCALE_SINGLE)
    return fail(c, CVR_ERR_UNSUPPORTED, "cvr_batch_create: multiscaling is per frame, not batched (turn it off)");
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaStreamSynchronize(c->stream));
  std::unique_ptr<cvr_batch> b(new cvr_batch());
  b->ctx = c;
  b->n_jobs = n_jobs;
  // longest jobs first within each method group
  std::vector<int> order(n_jobs);
  std::iota(order.begin(), order.end(), 0);
  // longest jobs first; among equal costs, jobs of one volume, method and
  // walk axis together, so that consecutive jobs share their tables in L2
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const double cx = job_cost(jobs[x], c), cy = job_cost(jobs[y], c);
    if (cx != cy) return cx > cy;
    if (jobs[x].volume != jobs[y].volume) return jobs[x].volume < jobs[y].volume;
    if (jobs[x].method != jobs[y].method) return jobs[x].method < jobs[y].method;
    return job_walk_axis(jobs[x]) < job_walk_axis(jobs[y]);
  });
  CK(c, cudaMalloc((void**)&b->d_stats, sizeof(unsigned long long) * 3 * n_jobs));
  std::vector<BatchExtJob> ext;
  std::vector<int> ext_slot;
  double slot_vmax[CVR_MAX_VOLUMES] = {};
  bool all_compact = c->compact_sat;
  std::vector<std::vector<float4>> tables;
  std::vector<SurLaunch> sur;  // the surrogate jobs in launches of up to kSurLaunchJobs
  unsigned long long sur_positions = 0;
  const int keep = c->cur_slot;
  cvr_status st = CVR_OK;
  for (int oi = 0; oi < n_jobs && st == CVR_OK; ++oi) {
    const int i = order[oi];
    const cvr_job& j = jobs[i];
    select_slot(c, j.volume);
    FrameArgs f;
    st = frame_args(c, &j.camera, j.params, j.out_rgba_dev, j.width, j.height, &f);
    if (st != CVR_OK) break;
    st = grad_args(c, j.method, &j.light, &f);
    if (st != CVR_OK) break;
    f.stats = b->d_stats + 3 * (size_t)i;
    if (j.method == CVR_METHOD_EXTINCTION) {
      BatchExtJob J{};
      const ShadowBoxTable* table = nullptr;
      double vmax = 0.0;
      st = ext_args(c, static_cast<const cvr_ext_params*>(j.params), &j.light, f, &J.e, &table, &vmax);
      if (st != CVR_OK) break;
      if (vmax > 0.0) slot_vmax[j.volume] = std::max(slot_vmax[j.volume], vmax);
      else all_compact = false;
      ext_slot.push_back(j.volume);
      J.f = f;
      J.blocks_x = (unsigned)((j.width + f.tile_w - 1) / f.tile_w);
      J.first_block = b->ext_blocks;
      b->ext_blocks += J.blocks_x * (unsigned)((j.height + f.tile_h - 1) / f.tile_h);
      std::vector<float4> t;
      if (table) {
        J.tn = table->n; J.tax = table->axis; J.tiw = table->interval; J.tvmin = table->vmin; J.tvmax = table->vmax;
        t.assign(table->lo, table->lo + table->n);
        t.insert(t.end(), table->hi, table->hi + table->n);
        if (table->aligned) t.insert(t.end(), table->tx, table->tx + table->n);
        b->ext_max_table = std::max(b->ext_max_table, table->n);
      }
      tables.push_back(std::move(t));
      ext.push_back(J);
    } else {
      SurJob J{};
      bool tex = false;
      st = sur_job_args(c, static_cast<const cvr_gt_params*>(j.params), &j.light, &J.a, &tex);
      if (st != CVR_OK) break;
      if (!sur.empty() && tex != b->sur_tex) { st = fail(c, CVR_ERR_INVALID_ARG, "cvr_batch_create: mixed sampling"); break; }
      b->sur_tex = tex;
      J.f = f;
      const SurSpiral o = sur_spiral(f);
      J.cx = o.cx;
      J.cy = o.cy;
      J.tiles_x = (j.width + 7) / 8;
      J.tiles_y = (j.height + 3) / 4;
      if (sur.empty() || sur.back().n_jobs == kSurLaunchJobs) {
        sur.emplace_back();
        std::memset(&sur.back(), 0, sizeof(SurLaunch));
        sur_positions = 0;
      }
      SurLaunch& L = sur.back();
      J.first_tile = (unsigned)sur_positions;
      sur_positions += o.positions;
      if (sur_positions * 32ull > 0xFFFFFFF0ull) {
        st = fail(c, CVR_ERR_UNSUPPORTED, "cvr_batch_create: more than 2^32 surrogate rays in one launch");
        break;
      }
      L.total = (unsigned)(sur_positions * 32ull);
      L.jobs[L.n_jobs++] = J;
      ++b->n_sur;
    }
  }
  // Compact SATs owned by the batch (a later frame may rebuild the context's
  // own at another fixed point): one per slot, at the largest region of its jobs
  if (st == CVR_OK && all_compact && !ext.empty()) {
    float inv[CVR_MAX_VOLUMES] = {};
    uint4* tab[CVR_MAX_VOLUMES] = {};
    for (int v = 0; v < CVR_MAX_VOLUMES && st == CVR_OK && all_compact; ++v) {
      if (slot_vmax[v] <= 0.0) continue;
      select_slot(c, v);
      int F;
      std::vector<unsigned> q;
      if (!compact_plan(c->sat_ext, slot_vmax[v], &F, &q)) { all_compact = false; break; }
      const size_t cells = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
      if (cells >= kCompactMaxCells) { all_compact = false; break; }
      uint4* d = nullptr;
      cudaError_t e = cudaMalloc((void**)&d, cells * sizeof(uint4));
      if (e == cudaErrorMemoryAllocation) { cudaGetLastError(); all_compact = false; break; }  // int64 tables
      if (e != cudaSuccess) { st = cuda_fail(c, e, "cvr_batch_create: compact SAT"); break; }
      b->sat32.push_back(d);
      st = build_compact_sat(c, q, d);
      if (st == CVR_ERR_OUT_OF_MEMORY) { st = CVR_OK; all_compact = false; break; }
      tab[v] = d;
      inv[v] = (float)std::ldexp(1.0, -F);
    }
    if (st == CVR_OK && all_compact) {
      for (size_t k = 0; k < ext.size(); ++k) {
        ext[k].e.sat.sat32 = tab[ext_slot[k]];
        ext[k].e.sat.inv_scale32 = inv[ext_slot[k]];
      }
      b->ext_compact = true;
      // walk tables of these compact tables, one per (slot, walk axis, box
      // depth) that the jobs with an aligned directional table use (a job's
      // table holds its texel offsets after lo and hi when it is aligned)
      for (size_t k = 0; k < ext.size() && st == CVR_OK && c->walk_tables; ++k) {
        BatchExtJob& J = ext[k];
        if (J.tn <= 0 || tables[k].size() != 3 * (size_t)J.tn) continue;
        const int slot = ext_slot[k], axis = J.tax, w = (int)std::nearbyint(J.e.interval);
        if (w < 1 || w > 1023) continue;
        const long long key = ((long long)slot * 3 + axis) * 1024 + w;
        uint4* d = nullptr;
        for (size_t i = 0; i < b->walk_keys.size(); ++i)
          if (b->walk_keys[i] == key) d = b->walks[i];
        if (!d) {
          select_slot(c, slot);
          const int sx = c->nx + 2, sy = c->ny + 2, sz = c->nz + 2;
          cudaError_t e = cudaMalloc((void**)&d, (size_t)sx * sy * sz * 2 * sizeof(uint4));
          if (e == cudaErrorMemoryAllocation) { cudaGetLastError(); continue; }  // this job reads the quads
          if (e != cudaSuccess) { st = cuda_fail(c, e, "cvr_batch_create: walk table"); break; }
          b->walks.push_back(d);
          b->walk_keys.push_back(key);
          e = launch_sat_walk(tab[slot], d, sx, sy, sz, axis, w, c->stream);
          if (e != cudaSuccess) { st = cuda_fail(c, e, "cvr_batch_create: walk table"); break; }
        }
        J.e.walk = WalkView{d, axis, w};
      }
    }
  }
  select_slot(c, keep);
  if (st != CVR_OK) return st;
  if (!sur.empty() && (!c->mlp || !c->mlp->err)) return fail(c, CVR_ERR_NOT_READY, "cvr_batch_create: no network");
  b->ext_variant = c->variant;
  b->ext_threads = (c->tile_w / 8) * (c->tile_h / 4) * 32;
  b->n_ext = (int)ext.size();
  if (b->n_ext) {
    // shadow tables: one region per job, pointers patched in
    size_t total = 0;
    for (auto& t : tables) total += t.size();
    if (total) {
      CK(c, cudaMalloc((void**)&b->d_tables, sizeof(float4) * total));
      size_t off = 0;
      for (size_t k = 0; k < ext.size(); ++k) {
        if (tables[k].empty()) continue;
        CK(c, cudaMemcpy(b->d_tables + off, tables[k].data(), sizeof(float4) * tables[k].size(), cudaMemcpyHostToDevice));
        ext[k].tlo = b->d_tables + off;
        ext[k].thi = b->d_tables + off + ext[k].tn;
        ext[k].ttx = tables[k].size() == 3 * (size_t)ext[k].tn ? b->d_tables + off + 2 * ext[k].tn : nullptr;
        off += tables[k].size();
      }
    }
    for (const BatchExtJob& J : ext)
      if (!J.e.sat.sat32 && !J.e.sat.sat) return fail(c, CVR_ERR_NOT_READY, "cvr_batch_create: a job without a SAT");
    b->ext_aligned = true;
    for (const BatchExtJob& J : ext)
      if (!J.ttx || !(J.e.ao_aligned || !J.e.apply_occ)) b->ext_aligned = false;
    CK(c, cudaMalloc((void**)&b->d_ext, sizeof(BatchExtJob) * ext.size()));
    CK(c, cudaMemcpy(b->d_ext, ext.data(), sizeof(BatchExtJob) * ext.size(), cudaMemcpyHostToDevice));
  }
  const size_t n_counters = 1 + sur.size();
  CK(c, cudaMalloc((void**)&b->d_counters, sizeof(unsigned int) * n_counters));
  // capture: counter and statistics resets, then the persistent launches
  cudaGraph_t g = nullptr;
  CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  cudaError_t e = cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned int) * n_counters, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_stats, 0, sizeof(unsigned long long) * 3 * n_jobs, c->stream);
  if (e == cudaSuccess && b->n_ext)
    e = launch_batch_extinction(b->d_ext, b->n_ext, b->ext_blocks, b->d_counters, c->tf_n, b->ext_max_table,
                                b->ext_threads, b->ext_variant, b->ext_compact, b->ext_aligned, c->stream);
  for (size_t k = 0; k < sur.size() && e == cudaSuccess; ++k)
    e = launch_batch_surrogate(sur[k], c->tf_n, b->sur_tex, b->ext_variant, b->d_counters + 1 + k, c->mlp->err,
                               c->stream);
  cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(c, e != cudaSuccess ? e : e2, "cvr_batch_create: capture");
  }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cvr_batch_create: graph instantiate");
  *out = b.release();
  return CVR_OK;
}

cvr_status cvr_batch_run(cvr_batch* b) {
  if (!b || !b->ctx) return CVR_ERR_INVALID_ARG;
  cvr_ctx* c = b->ctx;
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaGraphLaunch(b->graph, c->stream));
  return CVR_OK;
}

cvr_status cvr_batch_job_stats(cvr_batch* b, int job, cvr_frame_stats* out) {
  if (!b || !b->ctx || !out || job < 0 || job >= b->n_jobs) return CVR_ERR_INVALID_ARG;
  cvr_ctx* c = b->ctx;
  CK(c, cudaSetDevice(c->device));
  unsigned long long h[3];
  CK(c, cudaMemcpyAsync(h, b->d_stats + 3 * (size_t)job, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  out->samples = h[0];
  out->shaded_samples = h[1];
  out->aux_fetches = h[2];
  out->kernel_ms = 0.0f;
  return mlp_check_err(c);
}

void cvr_batch_destroy(cvr_batch* b) {
  if (!b) return;
  if (b->ctx) {
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
  }
  delete b;
}

}  // extern "C"
