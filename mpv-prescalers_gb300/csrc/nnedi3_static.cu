// NNEDI3 for callers that cannot allocate device memory: pz_nnedi3_run_static.
//
// Doubling both axes takes two passes with a row-doubled plane in between
// (2H x W).  pz_run gets that plane from opts->scratch or allocates it
// stream-ordered.  Some hosts may not allocate while they render a frame:
// a player's render callback that runs against a display deadline (an
// allocation can block on the driver), a host that gives the library a
// fixed device-memory budget up front, or a caller inside a region where
// its own allocator must not be re-entered.  This entry point takes the
// intermediate plane from a fixed array compiled into the library instead
// and calls no allocating routine of any kind.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds its PZ_STATIC_SCRATCH_BYTES until the process exits.  Host
// code cannot pass the variable's name to a kernel (on the host it is only a
// stand-in, not a device address), so the first call on each device looks
// the device address up with cudaGetSymbolAddress while that device is
// current, and later calls reuse it.  Make that first call before any stream
// capture.  All calls share the one array and it keeps whatever the last
// call left in it: nothing in it has to start at zero (the row pass writes
// the whole intermediate before the column pass reads it).  A bounded
// device-side wait that runs out is reported in the library's device error
// word (a __device__ variable as well), which pz_check_device_error reads and
// clears.  Calls that overlap on the GPU (several streams, or several threads
// without ordering between them) race on the array; order them.
#include <cstring>
#include <mutex>

#include "../../include/prescale.h"
#include "kernels.h"
#include "model.h"

namespace {

__device__ __align__(256) unsigned char g_static_scratch[PZ_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
struct StaticAddr {
  void* scratch;
  int* err;
};
std::mutex g_addr_mu;
StaticAddr g_addr[kMaxDevices];  // resolved on the first call on each device

// Device addresses of the static array and of the error word on the current
// device.
int resolve_static(StaticAddr* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pz::set_error(PZ_EIO, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return pz::set_error(PZ_ENOTSUP, "device %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev].scratch) {
    void* s = nullptr;
    e = cudaGetSymbolAddress(&s, g_static_scratch);
    if (e != cudaSuccess) return pz::set_error(PZ_EIO, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    int* w = pz::device_error_word();
    if (!w) return pz::set_error(PZ_EIO, "device error word: cudaGetSymbolAddress failed");
    g_addr[dev].scratch = s;
    g_addr[dev].err = w;
  }
  *out = g_addr[dev];
  return PZ_OK;
}

int check(const pz_plane* p, const char* what, bool pairs) {
  if (!p || !p->data) return pz::set_error(PZ_EINVAL, "%s: null plane", what);
  if (p->width <= 0 || p->height <= 0 || p->pitch < p->width)
    return pz::set_error(PZ_EINVAL, "%s: bad size %dx%d pitch %d", what, p->width, p->height, p->pitch);
  if (p->dtype != PZ_F32 && p->dtype != PZ_F16) return pz::set_error(PZ_EINVAL, "%s: unknown dtype", what);
  const size_t es = p->dtype == PZ_F32 ? 4 : 2;
  const uintptr_t a = reinterpret_cast<uintptr_t>(p->data);
  if (a % es || (pairs && (a % (2 * es) || p->pitch % 2)))
    return pz::set_error(PZ_EINVAL, "%s: misaligned base or pitch", what);
  return PZ_OK;
}

}  // namespace

extern "C" int pz_nnedi3_run_static(const pz_model* m, const pz_plane* in, pz_plane* out, const pz_opts* o,
                                    void* stream) {
  if (!m || m->family != PZ_NNEDI3) return pz::set_error(PZ_EINVAL, "pz_nnedi3_run_static needs an NNEDI3 model");
  const int ax = (o && o->nnedi3_axes) ? o->nnedi3_axes : 3;
  if (ax < 1 || ax > 3) return pz::set_error(PZ_EINVAL, "nnedi3_axes must be 1, 2 or 3");
  int rc;
  if ((rc = check(in, "in", false)) || (rc = check(out, "out", (ax & 2) != 0))) return rc;
  if (out->dtype != in->dtype) return pz::set_error(PZ_EINVAL, "in and out must share one dtype");
  if ((rc = pz::check_opts(o, in->dtype))) return rc;
  const int W = in->width, H = in->height, dt = in->dtype;
  const size_t es = dt == PZ_F32 ? 4 : 2;
  const int OW = (ax & 2) ? 2 * W : W, OH = (ax & 1) ? 2 * H : H;
  if (out->width != OW || out->height != OH)
    return pz::set_error(PZ_EINVAL, "output must be %dx%d, got %dx%d", OW, OH, out->width, out->height);
  const size_t need = ax == 3 ? (size_t)2 * H * W * es : 0;
  if (need > PZ_STATIC_SCRATCH_BYTES)
    return pz::set_error(PZ_EINVAL,
                         "a %dx%d %s frame needs %zu bytes of intermediate plane; the static array holds %u "
                         "(2 * width * height * element size must fit)",
                         W, H, dt == PZ_F32 ? "FP32" : "FP16", need, (unsigned)PZ_STATIC_SCRATCH_BYTES);
  StaticAddr addr;
  if ((rc = resolve_static(&addr))) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const bool fast = o && o->precision == PZ_PREC_FAST && pz::nnedi3_tc_supported(m->nns, m->win_h);
  pz::NnArgs a{};
  a.nns = m->nns;
  a.win_h = m->win_h;
  a.wts = m->d_wts;
  a.cs = m->d_cs;
  a.bias = m->d_bias;
  a.wts_h = m->d_wts_h;
  a.err = addr.err;
  auto pass = [&](bool xpass, const void* src, int sw, int sh, int spitch, void* dst, int dpitch) {
    a.in = src;
    a.in_pitch = spitch;
    a.out = dst;
    a.out_pitch = dpitch;
    a.W = sw;
    a.H = sh;
    return fast ? pz::launch_nnedi3_tc(a, xpass, dt, s) : pz::launch_nnedi3_simt(a, xpass, dt, s);
  };
  if (ax == 3) {
    rc = pass(false, in->data, W, H, in->pitch, addr.scratch, W);
    if (!rc) rc = pass(true, addr.scratch, W, 2 * H, W, out->data, out->pitch);
  } else if (ax == 1) {
    rc = pass(false, in->data, W, H, in->pitch, out->data, out->pitch);
  } else {
    rc = pass(true, in->data, W, H, in->pitch, out->data, out->pitch);
  }
  if (rc) return pz::set_error(rc, "NNEDI3 launch configuration not supported");
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pz::set_error(PZ_EIO, "kernel launch: %s", cudaGetErrorString(e));
  return PZ_OK;
}
