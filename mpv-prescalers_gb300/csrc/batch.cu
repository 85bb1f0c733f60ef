// Batched execution: many frames (any sizes) of many RAVU models in one
// persistent launch, plus the NNEDI3 jobs of the batch.
//
// The reference runs one shader dispatch per pass per frame; a player with
// several streams issues them back to back.  Here a plan uploads one table of
// job descriptors to caller-provided device memory; each launch then
//   phase 0: one persistent kernel per plane dtype runs every first-pass tile
//            of every job (ravu-lite, ravu-3x, ravu-zoom, ravu int11), CTAs
//            pulling tile numbers from a device counter;
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
#include "batch_kernel.cuh"

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

int* device_error_word();
}  // namespace pz

// Host plan: what one launch enqueues.
struct pz_batch {
  struct Group {  // one persistent launch
    int dtype;
    int phase;
    int hset;       // program set: 1 = the fast form's FP16-texel programs
    int first_job;  // index into the device table
    int n_jobs;
    int total_tiles;
    int counter;    // index of its counter int
  };
  std::vector<Group> groups;
  std::vector<pz_job> nnedi3;  // run as their own launches
  void* work = nullptr;
  int n_counters = 0;
  int ctas_per_sm = 0;         // 0 = as many as fit
  int grid[2][2] = {{0, 0}, {0, 0}};  // per dtype and program set
};

namespace {

int build_tables(const pz_job* jobs, int n, std::vector<pz::DevJob>* table, pz_batch* plan, int phase_filter) {
  (void)phase_filter;
  for (int dt = 0; dt < 2; dt++) {
    for (int phase = 0; phase < 2; phase++) {
     for (int hset = 0; hset < 2; hset++) {
      pz_batch::Group g{dt, phase, hset, (int)table->size(), 0, 0, plan->n_counters};
      for (int i = 0; i < n; i++) {
        const pz_job& j = jobs[i];
        const pz_model* m = j.model;
        if (m->family == PZ_NNEDI3) continue;
        if (j.in[0].dtype != dt) continue;
        if (phase == 1 && m->family != PZ_RAVU) continue;
        if (pz::fast_half_lut(m, j.opts.precision) != (hset == 1)) continue;
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
        a.ar = m->ar;
        a.keys = nullptr;
        a.err = pz::device_error_word();
        a.kp = m->kp;
        d.prog = pz::prog_of(m, j.opts.precision) + (phase == 1 ? pz::kLattice0 - pz::kInt110 : 0);
        const bool zoom = m->family == PZ_RAVU_ZOOM;
        const int tw = ((zoom ? a.OW : a.W) + pz::kTileW - 1) / pz::kTileW;
        const int th = ((zoom ? a.OH : a.H) + pz::kTileH - 1) / pz::kTileH;
        d.tiles_w = tw;
        d.first_tile = g.total_tiles;
        g.total_tiles += tw * th;
        table->push_back(d);
        g.n_jobs++;
      }
      if (g.n_jobs) {
        plan->groups.push_back(g);
        plan->n_counters++;
      }
     }
    }
  }
  return PZ_OK;
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
  if (j.opts.precision < PZ_PREC_FP32 || j.opts.precision > PZ_PREC_MPV)
    return pz::set_error(PZ_EINVAL, "job %d: unknown precision %d", idx, j.opts.precision);
  if (j.opts.precision == PZ_PREC_MPV && j.in[0].dtype != PZ_F16)
    return pz::set_error(PZ_EINVAL, "job %d: the mpv form takes FP16 planes", idx);
  const int W = j.in[0].width, H = j.in[0].height, OW = j.out[0].width, OH = j.out[0].height;
  const size_t es = j.in[0].dtype == PZ_F32 ? 4 : 2;
  switch (m->family) {
    case PZ_RAVU_LITE:
    case PZ_RAVU:
    case PZ_NNEDI3:
      if (m->family == PZ_NNEDI3) break;  // checked by pz_run at launch
      if (OW != 2 * W || OH != 2 * H) return pz::set_error(PZ_EINVAL, "job %d: output must be 2x the input", idx);
      if (m->family == PZ_RAVU_LITE &&
          ((reinterpret_cast<uintptr_t>(j.out[0].data) % (2 * es)) || (j.out[0].pitch % 2)))
        return pz::set_error(PZ_EINVAL, "job %d: ravu-lite output must be 2-element aligned", idx);
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
  size_t n = 0;
  for (int i = 0; i < n_jobs; i++)
    if (jobs[i].model && jobs[i].model->family != PZ_NNEDI3) n += jobs[i].model->family == PZ_RAVU ? 2 : 1;
  return pz::align256(8 * sizeof(int)) + n * sizeof(pz::DevJob);
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
  build_tables(jobs, n_jobs, &table, plan, 0);
  for (int i = 0; i < n_jobs; i++)
    if (jobs[i].model->family == PZ_NNEDI3) plan->nnedi3.push_back(jobs[i]);
  plan->work = work;
  plan->ctas_per_sm = ctas_per_sm;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!table.empty()) {
    cudaError_t e = cudaMemcpyAsync(static_cast<char*>(work) + pz::align256(8 * sizeof(int)), table.data(),
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
  for (int dt = 0; dt < 2; dt++) {
    for (int h = 0; h < 2; h++) {
      int fit = dt == 0 ? (h ? pz::batch_fit_f32h() : pz::batch_fit_f32())
                        : (h ? pz::batch_fit_f16h() : pz::batch_fit_f16());
      if (fit < 1) fit = 1;
      const int per = ctas_per_sm > 0 ? std::min(ctas_per_sm, fit) : fit;
      plan->grid[dt][h] = per * sms;
    }
  }
  *out = plan;
  return PZ_OK;
}

int pz_batch_launch(const pz_batch* plan, void* stream) {
  if (!plan) return pz::set_error(PZ_EINVAL, "null plan");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* counters = static_cast<int*>(plan->work);
  const pz::DevJob* table =
      reinterpret_cast<const pz::DevJob*>(static_cast<char*>(plan->work) + pz::align256(8 * sizeof(int)));
  if (!plan->groups.empty()) {
    cudaError_t e = cudaMemsetAsync(counters, 0, 8 * sizeof(int), s);
    if (e != cudaSuccess) return pz::set_error(PZ_EIO, "clearing the work counters: %s", cudaGetErrorString(e));
  }
  for (const auto& g : plan->groups) {  // phase 0 groups come before phase 1 of the same dtype
    const int grid = std::min(plan->grid[g.dtype][g.hset], g.total_tiles);
    auto* launch = g.dtype == PZ_F32 ? (g.hset ? pz::launch_batch_f32h : pz::launch_batch_f32)
                                     : (g.hset ? pz::launch_batch_f16h : pz::launch_batch_f16);
    launch(table + g.first_job, g.n_jobs, g.total_tiles, counters + g.counter, grid, s);
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
