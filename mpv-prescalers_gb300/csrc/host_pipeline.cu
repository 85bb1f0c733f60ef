// Frames in host memory: pz_run_host / pz_run_host_work_bytes.
//
// A host that decodes in software holds its frames in host memory.  This
// entry point runs a model's chain over N such frames with the transfers of
// neighbouring frames under each frame's kernels: frame i is copied to the
// device on a copy stream, run on the caller's stream and copied back on a
// second copy stream, through kDepth rotating device slots carved from the
// caller's work buffer.  Events order each slot's reuse (its previous frame
// must have left the device before the next one lands), so no call waits on
// the host; the caller's stream completes after the last frame is back.
// Calls on different caller streams take different copy-stream pairs (a
// small pool per device), so the results of two models' calls in flight
// together leave the device as each frame is done instead of one call's
// after the other's.
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "../../include/prescale.h"
#include "model.h"

namespace {

constexpr int kDepth = 3;        // device slots in flight (one per stream)
constexpr int kMaxDevices = 64;
constexpr int kPairs = 4;        // copy-stream pairs per device

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
size_t elem(int dtype) { return dtype == PZ_F32 ? 4 : 2; }

struct Layout {
  size_t in_bytes, out_bytes, scratch_bytes, slot_bytes;
  int out_w, out_h, n_planes;
};

int layout(const pz_model* m, int w, int h, int dtype, const pz_opts* o, Layout* L) {
  pz_query_result r;
  const int rc = pz_query(m, w, h, dtype, o, &r);
  if (rc) return rc;
  L->n_planes = r.n_planes;
  L->out_w = r.out_width;
  L->out_h = r.out_height;
  L->in_bytes = (size_t)r.n_planes * w * h * elem(dtype);
  L->out_bytes = (size_t)r.n_planes * r.out_width * r.out_height * elem(dtype);
  L->scratch_bytes = r.scratch_bytes;
  L->slot_bytes = align256(L->in_bytes) + align256(L->out_bytes) + align256(L->scratch_bytes);
  return PZ_OK;
}

// kPairs pairs of copy streams per device, created on first use and kept
// for the process (non-blocking: they never wait on the legacy default
// stream).  A caller stream keeps the pair it was first given (pairs are
// handed out in turn), so its calls stay ordered on one pair.
std::mutex g_stream_mu;
cudaStream_t g_copy[kMaxDevices][kPairs][2];
std::unordered_map<cudaStream_t, int> g_pair_of[kMaxDevices];
int g_next_pair[kMaxDevices];

int copy_streams(cudaStream_t caller, cudaStream_t* in, cudaStream_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pz::set_error(PZ_EIO, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return pz::set_error(PZ_ENOTSUP, "device %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lk(g_stream_mu);
  auto& pairs = g_pair_of[dev];
  auto it = pairs.find(caller);
  int p;
  if (it != pairs.end()) {
    p = it->second;
  } else {
    if (pairs.size() >= 1024) pairs.clear();  // forget streams long gone (a pairing, not a resource)
    p = g_next_pair[dev]++ % kPairs;
    pairs.emplace(caller, p);
  }
  for (int k = 0; k < 2; k++) {
    if (!g_copy[dev][p][k]) {
      e = cudaStreamCreateWithFlags(&g_copy[dev][p][k], cudaStreamNonBlocking);
      if (e != cudaSuccess) return pz::set_error(PZ_EIO, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
  }
  *in = g_copy[dev][p][0];
  *out = g_copy[dev][p][1];
  return PZ_OK;
}

}  // namespace

extern "C" size_t pz_run_host_work_bytes(const pz_model* m, int width, int height, int dtype, const pz_opts* o) {
  Layout L;
  if (!m || layout(m, width, height, dtype, o, &L)) return 0;
  return kDepth * L.slot_bytes;
}

extern "C" int pz_run_host(const pz_model* m, const void* host_in, void* host_out, int n_frames, int width,
                           int height, int dtype, const pz_opts* o, void* work, size_t work_bytes, int flags,
                           void* stream) {
  if (!m || !host_in || !host_out || !work) return pz::set_error(PZ_EINVAL, "null argument");
  if (n_frames <= 0) return pz::set_error(PZ_EINVAL, "n_frames %d", n_frames);
  Layout L;
  int rc = layout(m, width, height, dtype, o, &L);
  if (rc) return rc;
  // one device slot per frame in flight: fewer frames than slots need fewer
  const int depth = n_frames < kDepth ? n_frames : kDepth;
  if (work_bytes < depth * L.slot_bytes)
    return pz::set_error(PZ_EINVAL, "work of %zu bytes, %d frames in flight need %zu", work_bytes, depth,
                         depth * L.slot_bytes);
  if (reinterpret_cast<uintptr_t>(work) % 256) return pz::set_error(PZ_EINVAL, "work must be 256-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream), s_in, s_out;
  if ((rc = copy_streams(s, &s_in, &s_out))) return rc;

  cudaEvent_t start, fin, copied[kDepth], done[kDepth], drained[kDepth];
  cudaEvent_t* all[] = {&start, &fin};
  int made = 0;
  cudaError_t e = cudaSuccess;
  for (cudaEvent_t* ev : all) {
    if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess) break;
    made++;
  }
  int made_slots = 0;
  for (int b = 0; b < kDepth && e == cudaSuccess; b++) {
    if ((e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming)) != cudaSuccess) break;
    if ((e = cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming)) != cudaSuccess) {
      cudaEventDestroy(copied[b]);
      break;
    }
    if ((e = cudaEventCreateWithFlags(&drained[b], cudaEventDisableTiming)) != cudaSuccess) {
      cudaEventDestroy(copied[b]);
      cudaEventDestroy(done[b]);
      break;
    }
    made_slots++;
  }
  auto release = [&]() {  // events still pending are released once they complete
    for (int k = 0; k < made; k++) cudaEventDestroy(*all[k]);
    for (int b = 0; b < made_slots; b++) {
      cudaEventDestroy(copied[b]);
      cudaEventDestroy(done[b]);
      cudaEventDestroy(drained[b]);
    }
  };
  if (e != cudaSuccess) {
    release();
    return pz::set_error(PZ_EIO, "cudaEventCreate: %s", cudaGetErrorString(e));
  }

  const size_t es = elem(dtype);
  const char* hin = static_cast<const char*>(host_in);
  char* hout = static_cast<char*>(host_out);
  char* slots = static_cast<char*>(work);
  pz_opts opts = o ? *o : pz_opts{};
  // unless the caller vouches that `work` is idle, the copies wait for the
  // work queued earlier on the caller's stream (which may still use it)
  if (!(flags & PZ_HOST_WORK_IDLE)) {
    e = cudaEventRecord(start, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s_in, start, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s_out, start, 0);
  }
  for (int i = 0; i < n_frames && e == cudaSuccess && rc == PZ_OK; i++) {
    const int b = i % depth;
    char* d_in = slots + b * L.slot_bytes;
    char* d_out = d_in + align256(L.in_bytes);
    char* d_scr = d_out + align256(L.out_bytes);
    if (i >= depth) e = cudaStreamWaitEvent(s_in, drained[b], 0);  // slot b's last frame has left
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_in, hin + (size_t)i * L.in_bytes, L.in_bytes, cudaMemcpyHostToDevice, s_in);
    if (e == cudaSuccess) e = cudaEventRecord(copied[b], s_in);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, copied[b], 0);
    if (e != cudaSuccess) break;
    pz_plane pin[3], pout[3];
    for (int c = 0; c < L.n_planes; c++) {
      pin[c] = pz_plane{d_in + (size_t)c * width * height * es, width, height, width, dtype};
      pout[c] = pz_plane{d_out + (size_t)c * L.out_w * L.out_h * es, L.out_w, L.out_h, L.out_w, dtype};
    }
    opts.scratch = L.scratch_bytes ? d_scr : nullptr;
    opts.scratch_bytes = L.scratch_bytes;
    rc = pz_run(m, pin, L.n_planes, pout, L.n_planes, &opts, s);  // slot b's output was drained before its input
    if (rc) break;
    e = cudaEventRecord(done[b], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s_out, done[b], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hout + (size_t)i * L.out_bytes, d_out, L.out_bytes, cudaMemcpyDeviceToHost, s_out);
    if (e == cudaSuccess) e = cudaEventRecord(drained[b], s_out);
  }
  // the caller's stream completes once every frame is back in host memory
  if (e == cudaSuccess) e = cudaEventRecord(fin, s_out);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, fin, 0);
  release();
  if (rc) return rc;
  if (e != cudaSuccess) return pz::set_error(PZ_EIO, "host pipeline: %s", cudaGetErrorString(e));
  return PZ_OK;
}
