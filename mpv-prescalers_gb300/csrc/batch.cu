// Batched execution: many frames (any sizes) of many RAVU models in a few
// persistent launches, plus the NNEDI3 jobs of the batch.
//
// The reference runs one shader dispatch per pass per frame; a player with
// several streams issues them back to back.  Here a plan uploads one table of
// job descriptors to caller-provided device memory, grouped by tile program
// (family, radius, channels, anti-ringing, LUT form) and plane dtype; each
// launch then runs
//   phase 0: per group, one persistent kernel of that program over every
//            first-pass tile of the group's frames (ravu-lite, ravu-3x,
//            ravu-zoom, ravu int11), CTAs pulling tile numbers from the
//            group's device counter -- register use and shared memory are the
//            program's own, as in a per-frame launch;
//   phase 1: the same for the ravu lattice pass (int10/int01), which reads
//            the int11 values phase 0 wrote;
//   NNEDI3 jobs are stream-ordered launches of their two passes.
// Launching only enqueues memsets and kernels, so a plan can be captured in a
// CUDA graph and replayed while its frames' buffers stay in place.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/prescale.h"
#include "model.h"
#include "ravu_tiles.cuh"

namespace pz {
namespace {

int prog_of(const pz_model* m, int precision) {
  const int R = m->radius, cm = m->channels, ar = m->ar != 0.0f;
  const bool h = fast_half_lut(m, precision);
  switch (m->family) {
    case PZ_RAVU_LITE: return (h ? kLiteH0 : kLite0) + (R - 2) * 2 + ar;
    case PZ_RAVU_3X: return (h ? kThreeXH0 : kThreeX0) + (R - 2) * 3 + cm;
    case PZ_RAVU: return kInt110 + (R - 2) * 3 + cm;
    case PZ_RAVU_ZOOM: return (h ? kZoomH0 : kZoom0) + (R - 2) * 6 + cm * 2 + ar;
  }
  return -1;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

}  // namespace pz

// Host plan: what one launch enqueues.
struct pz_batch {
  struct Group {  // one persistent launch: one program, one plane dtype
    int phase;
    int dtype;
    int prog;
    int first_job;    // index into the device table
    int n_jobs;
    int total_tiles;
    int grid;
    pz::PersistentOps ops;
  };
  std::vector<Group> groups;   // phase 0 groups, then phase 1
  std::vector<pz_job> nnedi3;  // run as their own launches
  void* work = nullptr;
  size_t table_offset = 0;     // the counters (one int per group) come first
};

namespace {

pz::PersistentOps ops_of(int prog, int dtype) {
  if (prog >= pz::kInt110 && prog < pz::kZoom0) return pz::persistent_ops_lattice(prog, dtype);
  if ((prog >= pz::kZoom0 && prog < pz::kLiteH0) || prog >= pz::kZoomH0) return pz::persistent_ops_zoom(prog, dtype);
  return pz::persistent_ops_lite(prog, dtype);
}

// Table entries of the RAVU jobs (one per job and phase), grouped by
// (phase, dtype, program) with each group's tile prefix sums.
int build_tables(const pz_job* jobs, int n, std::vector<pz::DevJob>* table, pz_batch* plan) {
  struct Entry {
    int phase, dtype, prog, job;
  };
  std::vector<Entry> entries;
  for (int i = 0; i < n; i++) {
    const pz_model* m = jobs[i].model;
    if (m->family == PZ_NNEDI3) continue;
    const int prog = pz::prog_of(m, jobs[i].opts.precision);
    entries.push_back({0, jobs[i].in[0].dtype, prog, i});
    if (m->family == PZ_RAVU) entries.push_back({1, jobs[i].in[0].dtype, prog + pz::kLattice0 - pz::kInt110, i});
  }
  std::stable_sort(entries.begin(), entries.end(), [](const Entry& a, const Entry& b) {
    if (a.phase != b.phase) return a.phase < b.phase;
    if (a.dtype != b.dtype) return a.dtype < b.dtype;
    return a.prog < b.prog;
  });
  for (size_t e = 0; e < entries.size(); e++) {
    const Entry& en = entries[e];
    if (plan->groups.empty() || plan->groups.back().phase != en.phase || plan->groups.back().dtype != en.dtype ||
        plan->groups.back().prog != en.prog) {
      pz_batch::Group g{};
      g.phase = en.phase;
      g.dtype = en.dtype;
      g.prog = en.prog;
      g.first_job = (int)table->size();
      g.ops = ops_of(en.prog, en.dtype);
      if (!g.ops.launch) return pz::set_error(PZ_ENOTSUP, "no persistent kernel for program %d", en.prog);
      plan->groups.push_back(g);
    }
    pz_batch::Group& g = plan->groups.back();
    const pz_job& j = jobs[en.job];
    const pz_model* m = j.model;
    pz::DevJob d{};
    pz::RavuArgs& a = d.a;
    const int C = m->channels == PZ_LUMA ? 1 : 3;
    for (int c = 0; c < C; c++) {
      a.in[c] = j.in[c].data;
      a.in_pitch[c] = j.in[c].pitch;
      a.out[c] = j.out[c].data;
      a.out_pitch[c] = j.out[c].pitch;
    }
    a.W = j.in[0].width;
    a.H = j.in[0].height;
    a.OW = j.out[0].width;
    a.OH = j.out[0].height;
    pz::select_lut(m, j.opts.precision, &a);
    a.i11 = m->family == PZ_RAVU ? static_cast<float*>(j.opts.scratch) : nullptr;
    a.ar = m->ar;
    a.keys = nullptr;
    a.err = pz::device_error_word();
    if (!a.err) return pz::set_error(PZ_EIO, "device error word: cudaGetSymbolAddress failed");
    a.kp = m->kp;
    d.prog = en.prog;
    const bool zoom = m->family == PZ_RAVU_ZOOM;
    const int tw = ((zoom ? a.OW : a.W) + pz::kTileW - 1) / pz::kTileW;
    const int th = ((zoom ? a.OH : a.H) + pz::kBatchTileRows - 1) / pz::kBatchTileRows;
    a.tile_rows = pz::kBatchTileRows;
    d.tiles_w = tw;
    d.first_tile = g.total_tiles;
    // interior tiles of jobs that ask for TMA staging come in as TMA boxes
    // (the maps live in the device table); a map the driver rejects leaves
    // the job on clamped loads
    a.staging = j.opts.staging;
    d.has_maps = j.opts.staging == 1 && g.ops.encode && g.ops.encode(&a, &d.maps) ? 1 : 0;
    g.total_tiles += tw * th;
    table->push_back(d);
    g.n_jobs++;
  }
  return PZ_OK;
}

// Table entries (= the most groups) of a job list.
size_t n_entries(const pz_job* jobs, int n_jobs) {
  size_t n = 0;
  for (int i = 0; i < n_jobs; i++)
    if (jobs[i].model && jobs[i].model->family != PZ_NNEDI3) n += jobs[i].model->family == PZ_RAVU ? 2 : 1;
  return n;
}

int validate_job(const pz_job& j, int idx) {
  if (!j.model) return pz::set_error(PZ_EINVAL, "job %d: null model", idx);
  const pz_model* m = j.model;
  const int C = m->channels == PZ_LUMA ? 1 : 3;
  if (j.n_planes != C) return pz::set_error(PZ_EINVAL, "job %d: model needs %d planes, got %d", idx, C, j.n_planes);
  for (int c = 0; c < C; c++) {
    const pz_plane &i = j.in[c], &o = j.out[c];
    if (!i.data || !o.data || i.width <= 0 || i.height <= 0 || i.pitch < i.width || o.pitch < o.width)
      return pz::set_error(PZ_EINVAL, "job %d plane %d: bad plane", idx, c);
    if (i.dtype != j.in[0].dtype || o.dtype != i.dtype || (i.dtype != PZ_F32 && i.dtype != PZ_F16))
      return pz::set_error(PZ_EINVAL, "job %d: all planes of a job must share one dtype", idx);
    if (i.width != j.in[0].width || i.height != j.in[0].height || o.width != j.out[0].width ||
        o.height != j.out[0].height)
      return pz::set_error(PZ_EINVAL, "job %d: planes differ in size", idx);
  }
  int rc;
  if ((rc = pz::check_opts(&j.opts, j.in[0].dtype))) return rc;
  const int W = j.in[0].width, H = j.in[0].height, OW = j.out[0].width, OH = j.out[0].height;
  const size_t es = j.in[0].dtype == PZ_F32 ? 4 : 2;
  switch (m->family) {
    case PZ_RAVU_LITE:
    case PZ_RAVU:
    case PZ_NNEDI3:
      if (m->family == PZ_NNEDI3) break;  // checked by pz_run at launch
      if (OW != 2 * W || OH != 2 * H) return pz::set_error(PZ_EINVAL, "job %d: output must be 2x the input", idx);
      for (int c = 0; c < C; c++)
        if ((reinterpret_cast<uintptr_t>(j.out[c].data) % (2 * es)) || (j.out[c].pitch % 2))
          return pz::set_error(PZ_EINVAL, "job %d: ravu / ravu-lite outputs must be 2-element aligned", idx);
      if (m->family == PZ_RAVU &&
          (!j.opts.scratch || j.opts.scratch_bytes < pz::lattice_scratch_bytes(m, W, H) ||
           reinterpret_cast<uintptr_t>(j.opts.scratch) % 4))
        return pz::set_error(PZ_EINVAL, "job %d: a ravu lattice job needs opts.scratch of %zu bytes (int11 plane)",
                             idx, pz::lattice_scratch_bytes(m, W, H));
      break;
    case PZ_RAVU_3X:
      if (OW != 3 * W || OH != 3 * H) return pz::set_error(PZ_EINVAL, "job %d: output must be 3x the input", idx);
      break;
    case PZ_RAVU_ZOOM:
      if (OW <= W || OH <= H) return pz::set_error(PZ_EINVAL, "job %d: ravu-zoom upscales only", idx);
      break;
    default:
      return pz::set_error(PZ_EINVAL, "job %d: unknown family", idx);
  }
  return PZ_OK;
}

}  // namespace

extern "C" {

size_t pz_batch_work_bytes(const pz_job* jobs, int n_jobs) {
  if (!jobs || n_jobs <= 0) return 0;
  const size_t n = n_entries(jobs, n_jobs);
  return pz::align256(n * sizeof(int)) + n * sizeof(pz::DevJob);
}

int pz_batch_create(const pz_job* jobs, int n_jobs, void* work, size_t work_bytes, int ctas_per_sm, void* stream,
                    pz_batch** out) {
  if (!jobs || n_jobs <= 0 || !out) return pz::set_error(PZ_EINVAL, "null or empty job list");
  *out = nullptr;
  int rc;
  for (int i = 0; i < n_jobs; i++)
    if ((rc = validate_job(jobs[i], i))) return rc;
  const size_t need = pz_batch_work_bytes(jobs, n_jobs);
  if (need && (!work || work_bytes < need))
    return pz::set_error(PZ_EINVAL, "work buffer of %zu bytes, batch needs %zu", work_bytes, need);
  pz_batch* plan = new (std::nothrow) pz_batch();
  if (!plan) return pz::set_error(PZ_ENOMEM, "host allocation failed");
  std::vector<pz::DevJob> table;
  if ((rc = build_tables(jobs, n_jobs, &table, plan))) {
    delete plan;
    return rc;
  }
  for (int i = 0; i < n_jobs; i++)
    if (jobs[i].model->family == PZ_NNEDI3) plan->nnedi3.push_back(jobs[i]);
  plan->work = work;
  plan->table_offset = pz::align256(n_entries(jobs, n_jobs) * sizeof(int));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!table.empty()) {
    cudaError_t e = cudaMemcpyAsync(static_cast<char*>(work) + plan->table_offset, table.data(),
                                    table.size() * sizeof(pz::DevJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the table is pageable host memory
    if (e != cudaSuccess) {
      delete plan;
      return pz::set_error(PZ_EIO, "uploading the job table: %s", cudaGetErrorString(e));
    }
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (auto& g : plan->groups) {
    int fit = g.ops.fit();
    if (fit < 1) fit = 1;
    const int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, fit) : fit;
    g.grid = std::min(per * sms, g.total_tiles);
  }
  *out = plan;
  return PZ_OK;
}

int pz_batch_launch(const pz_batch* plan, void* stream) {
  if (!plan) return pz::set_error(PZ_EINVAL, "null plan");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* counters = static_cast<int*>(plan->work);
  const pz::DevJob* table = reinterpret_cast<const pz::DevJob*>(static_cast<char*>(plan->work) + plan->table_offset);
  if (!plan->groups.empty()) {
    cudaError_t e = cudaMemsetAsync(counters, 0, plan->groups.size() * sizeof(int), s);
    if (e != cudaSuccess) return pz::set_error(PZ_EIO, "clearing the work counters: %s", cudaGetErrorString(e));
  }
  for (size_t i = 0; i < plan->groups.size(); i++) {  // phase 0 groups come before phase 1
    const auto& g = plan->groups[i];
    g.ops.launch(table + g.first_job, g.n_jobs, g.total_tiles, counters + i, g.grid, s);
  }
  for (const pz_job& j : plan->nnedi3) {
    int rc = pz_run(j.model, j.in, j.n_planes, const_cast<pz_plane*>(j.out), j.n_planes, &j.opts, stream);
    if (rc) return rc;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pz::set_error(PZ_EIO, "batch launch: %s", cudaGetErrorString(e));
  return PZ_OK;
}

void pz_batch_destroy(pz_batch* plan) { delete plan; }

int pz_batch_run(const pz_job* jobs, int n_jobs, void* work, size_t work_bytes, void* stream) {
  pz_batch* plan = nullptr;
  int rc = pz_batch_create(jobs, n_jobs, work, work_bytes, 0, stream, &plan);
  if (rc) return rc;
  rc = pz_batch_launch(plan, stream);
  pz_batch_destroy(plan);
  return rc;
}

}  // extern "C"
