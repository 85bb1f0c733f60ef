// C ABI of libprescale.so (declared in include/prescale.h): model upload,
// argument checking, dispatch to the kernels, thread-local error messages.
#include <cuda.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/prescale.h"
#include "async.cuh"
#include "kernels.h"
#include "model.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(PZ_EIO, "%s: %s", what, cudaGetErrorString(e));
}

template <typename T>
int upload(T** dst, const void* src, size_t bytes) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), bytes);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy");
  return PZ_OK;
}

// The device-side error word every kernel reports into (first failure wins,
// see kErr* in common.cuh).  A file-scope __device__ variable: nothing is
// allocated for it, so the first launch on a device may come inside stream
// capture.  Host code looks its device address up once per device.
__device__ int g_device_err;

constexpr int kMaxDevices = 64;
std::mutex g_err_mu;
int* g_err_words[kMaxDevices];  // device address of g_device_err, per device

size_t dtype_size(int dt) { return dt == PZ_F32 ? 4 : 2; }

// A bounded wait that nothing ever completes: the mbarrier is initialised for
// one arrival and never arrived at, no copy or MMA is issued.  The wait gives
// up after `limit_ns` and reports kErrWaitTimeout like every kernel does.
__global__ void wait_selftest_kernel(int* err, unsigned long long limit_ns) {
  __shared__ __align__(8) unsigned long long mbar;
  const uint32_t mb = pz::smem_u32(&mbar);
  if (threadIdx.x == 0) pz::mbar_init(mb, 1);
  __syncthreads();
  if (!__syncthreads_and(pz::mbar_wait_bounded(mb, 0u, limit_ns)) && threadIdx.x == 0)
    atomicCAS(err, 0, pz::kErrWaitTimeout);
}

// `pairs`: the plane is written with 2-wide vector stores, so its base and
// pitch must keep every even column 2-element aligned.
int check_plane(const pz_plane& p, const char* what, int idx, bool pairs) {
  if (!p.data) return fail(PZ_EINVAL, "%s[%d]: null data", what, idx);
  if (p.width <= 0 || p.height <= 0) return fail(PZ_EINVAL, "%s[%d]: bad size %dx%d", what, idx, p.width, p.height);
  if (p.pitch < p.width) return fail(PZ_EINVAL, "%s[%d]: pitch %d < width %d", what, idx, p.pitch, p.width);
  if (p.dtype != PZ_F32 && p.dtype != PZ_F16) return fail(PZ_EINVAL, "%s[%d]: unknown dtype %d", what, idx, p.dtype);
  const size_t es = dtype_size(p.dtype);
  if ((reinterpret_cast<uintptr_t>(p.data) % es) != 0)
    return fail(PZ_EINVAL, "%s[%d]: data not aligned to its element size", what, idx);
  if (pairs && ((reinterpret_cast<uintptr_t>(p.data) % (2 * es)) != 0 || (p.pitch % 2) != 0))
    return fail(PZ_EINVAL, "%s[%d]: this output is written in pixel pairs; base and pitch must be 2-element aligned",
                what, idx);
  return PZ_OK;
}

}  // namespace

namespace pz {
// Tensor map of one plane for 2-D TMA boxes of box_w x box_h texels.  False
// when the plane cannot be described (base or row pitch not 16-byte aligned,
// plane smaller than a box, driver entry point missing): callers then use
// clamped loads.
bool encode_plane_map(CUtensorMap* map, const void* base, int W, int H, int pitch, int dtype, int box_w,
                      int box_h) {
  typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                               const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<EncodeFn>(fn);
  });
  const size_t es = dtype == PZ_F32 ? 4 : 2;
  if (!encode || W < box_w || H < box_h || box_w > 256 || box_h > 256) return false;
  if (reinterpret_cast<uintptr_t>(base) % 16 || ((size_t)pitch * es) % 16) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * es};
  const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, dtype == PZ_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
                            2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int* device_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lk(g_err_mu);
  if (!g_err_words[dev]) {
    void* w = nullptr;
    if (cudaGetSymbolAddress(&w, g_device_err) != cudaSuccess) return nullptr;
    g_err_words[dev] = static_cast<int*>(w);
  }
  return g_err_words[dev];
}

int check_opts(const pz_opts* o, int dtype) {
  if (o && (o->precision < PZ_PREC_FP32 || o->precision > PZ_PREC_MPV))
    return set_error(PZ_EINVAL, "unknown precision %d", o->precision);
  if (o && o->precision == PZ_PREC_MPV && dtype != PZ_F16)
    return set_error(PZ_EINVAL, "the mpv form takes FP16 planes (the host's textures are rgba16f)");
  if (o && (o->staging < 0 || o->staging > 1))
    return set_error(PZ_EINVAL, "staging %d: 0 (clamped loads) or 1 (TMA boxes)", o->staging);
  if (o && o->tile_rows != 0 && o->tile_rows != 4 && o->tile_rows != 8 && o->tile_rows != 16)
    return set_error(PZ_EINVAL, "tile_rows %d: 0 (default), 4, 8 or 16", o->tile_rows);
  return PZ_OK;
}
}  // namespace pz

extern "C" {

int pz_version(void) { return PZ_ABI_VERSION; }

const char* pz_last_error(void) { return g_err.c_str(); }

int pz_model_create(const pz_model_desc* d, pz_model** out) {
  if (!d || !out) return fail(PZ_EINVAL, "null argument");
  *out = nullptr;
  pz_model* m = new (std::nothrow) pz_model();
  if (!m) return fail(PZ_ENOMEM, "host allocation failed");
  cudaGetDevice(&m->device);
  m->family = d->family;
  m->radius = d->radius;
  m->channels = d->channels;
  m->ar = d->ar_strength;
  int rc = PZ_OK;
  if (d->family == PZ_NNEDI3) {
    if (d->nns <= 0 || d->nns % 8 || d->win_w != 8 || (d->win_h != 4 && d->win_h != 6) || !d->weights_a ||
        !d->weights_b || !d->bias_a || !d->bias_b) {
      delete m;
      return fail(PZ_EINVAL, "bad NNEDI3 description (nns %d, window %dx%d)", d->nns, d->win_w, d->win_h);
    }
    m->nns = d->nns;
    m->win_w = d->win_w;
    m->win_h = d->win_h;
    const int T = d->win_w * d->win_h, n = d->nns;
    std::vector<float> w((size_t)n * 2 * T), cs((size_t)n * 2), bias((size_t)n * 2);
    const int KP = (T + 3 + 15) / 16 * 16;  // taps + (mean term, bias hi, bias lo), padded to a K step
    std::vector<__half> wh((size_t)n * 2 * KP, __float2half_rn(0.0f));
    for (int k = 0; k < n; k++) {
      double sa = 0, sb = 0;
      for (int t = 0; t < T; t++) {
        float a = d->weights_a[(size_t)t * n + k], b = d->weights_b[(size_t)t * n + k];
        w[((size_t)k * 2 + 0) * T + t] = a;
        w[((size_t)k * 2 + 1) * T + t] = b;
        sa += a;
        sb += b;
      }
      cs[2 * k] = (float)sa;
      cs[2 * k + 1] = (float)sb;
      bias[2 * k] = d->bias_a[k];
      bias[2 * k + 1] = d->bias_b[k];
    }
    // tensor-core operand B [2*nns][KP] FP16, chunk-major: chunk c of NC
    // neurons (NC = 32, or nns when below) is NC softmax-branch rows followed by
    // NC Elliott-branch rows.  Row = [weights (T taps), sum of the weights,
    // bias hi, bias lo, 0...]; against A rows [x_hat, mean*invstd, 1, 1, 0...]
    // the MMA yields the whole pre-activation <x,w>*invstd + b.  Softmax rows
    // are scaled by log2(e) so the epilogue takes exp2 directly.  Stored as
    // no-swizzle K-major core matrices (8 rows x 8 halves; K-neighbours 64
    // halves apart, 8-row groups 8*KP apart).
    const int NC = pz::nnedi3_tc_chunk(n);
    const double kLog2e = 1.4426950408889634;
    for (int r = 0; r < 2 * n; r++) {
      const int chunk = r / (2 * NC), within = r % (2 * NC);
      const int k = chunk * NC + within % NC, br = within / NC;
      const double scale = br == 0 ? kLog2e : 1.0;
      auto put = [&](int t, double v) {
        wh[(size_t)(r >> 3) * 8 * KP + (t >> 3) * 64 + (r & 7) * 8 + (t & 7)] = __float2half_rn((float)v);
      };
      double sum = 0.0;
      for (int t = 0; t < T; t++) {
        const double v = w[((size_t)k * 2 + br) * T + t];
        sum += v;
        put(t, v * scale);
      }
      const double b = (br == 0 ? d->bias_a[k] : d->bias_b[k]) * scale;
      const float bhi = __half2float(__float2half_rn((float)b));
      put(T, sum * scale);
      put(T + 1, bhi);
      put(T + 2, b - bhi);
    }
    if ((rc = upload(&m->d_wts, w.data(), w.size() * 4)) || (rc = upload(&m->d_cs, cs.data(), cs.size() * 4)) ||
        (rc = upload(&m->d_bias, bias.data(), bias.size() * 4)) ||
        (rc = upload(&m->d_wts_h, wh.data(), wh.size() * 2))) {
      pz_model_destroy(m);
      return rc;
    }
    *out = m;
    return PZ_OK;
  }
  if (d->family < PZ_RAVU_LITE || d->family > PZ_RAVU_3X) {
    delete m;
    return fail(PZ_EINVAL, "unknown family %d", d->family);
  }
  const int maxr = d->family == PZ_RAVU_ZOOM ? 3 : 4;
  if (d->radius < 2 || d->radius > maxr) {
    delete m;
    return fail(PZ_ENOTSUP, "radius %d not supported for family %d", d->radius, d->family);
  }
  if (d->channels < PZ_LUMA || d->channels > PZ_RGB || (d->family == PZ_RAVU_LITE && d->channels != PZ_LUMA)) {
    delete m;
    return fail(PZ_EINVAL, "bad channels %d for family %d", d->channels, d->family);
  }
  if (!d->lut || d->lut_rows <= 0 || d->lut_cols <= 0 || !d->grad_weights || d->n_grad <= 0 || d->n_grad > 36) {
    delete m;
    return fail(PZ_EINVAL, "bad LUT / gradient description");
  }
  const int n = d->family == PZ_RAVU_LITE || d->family == PZ_RAVU_3X ? 2 * d->radius - 1 : 2 * d->radius;
  const int pts = n <= 4 ? n * n : (n - 2) * (n - 2);
  if (d->n_grad != pts) {
    delete m;
    return fail(PZ_EINVAL, "%d gradient weights, window needs %d", d->n_grad, pts);
  }
  pz::KeyParams& kp = m->kp;
  {
    // gradient points in kernel order (px outer, py inner); where both
    // stencils of a point share one scale c, gwf = gw c^2
    const bool four = d->family == PZ_RAVU || d->family == PZ_RAVU_ZOOM;
    const int p0 = n <= 4 ? 0 : 1, p1 = n <= 4 ? n : n - 1;
    const double scale2[3] = {1.0, 0.25, 1.0 / 144.0};  // c^2 per stencil kind
    int i = 0;
    for (int px = p0; px < p1; px++)
      for (int py = p0; py < p1; py++, i++) {
        const int kx = pz::stencil_kind(n, four, px), ky = pz::stencil_kind(n, four, py);
        kp.gw[i] = (float)d->grad_weights[i];
        kp.gwf[i] = kx == ky ? (float)((double)kp.gw[i] * scale2[kx]) : kp.gw[i];
      }
  }
  kp.log2_mode = d->strength_log2;
  if (kp.log2_mode) {
    kp.log2_scale = d->strength_scale;
    kp.log2_max = (float)d->strength_max;
    kp.n_strength = d->strength_max + 1;
  } else {
    if (d->n_strength_thr != 2 && d->n_strength_thr != 3) {
      delete m;
      return fail(PZ_EINVAL, "need 2 or 3 strength thresholds");
    }
    kp.n_thr = d->n_strength_thr;
    for (int i = 0; i < kp.n_thr; i++) kp.thr[i] = d->strength_thr[i];
    kp.n_strength = kp.n_thr + 1;
  }
  kp.coh0 = d->coherence_thr[0];
  kp.coh1 = d->coherence_thr[1];
  kp.rows = 24 * kp.n_strength * 3;
  const int want_rows = d->family == PZ_RAVU_ZOOM ? kp.rows * 9 : kp.rows;
  if (d->lut_rows != want_rows) {
    delete m;
    return fail(PZ_EINVAL, "LUT has %d rows, key layout needs %d", d->lut_rows, want_rows);
  }
  const int S = n * n;
  int need_cols = 0;
  switch (d->family) {
    case PZ_RAVU_LITE: need_cols = (S + 1) / 2; break;
    case PZ_RAVU: need_cols = (S / 2 + 3) / 4; break;
    case PZ_RAVU_3X: need_cols = 2 * ((S + 1) / 2); break;
    case PZ_RAVU_ZOOM: need_cols = 9 * ((S / 2 + 3) / 4); break;
  }
  if (d->lut_cols != need_cols) {
    delete m;
    return fail(PZ_EINVAL, "LUT has %d columns, radius %d needs %d", d->lut_cols, d->radius, need_cols);
  }
  if (d->family == PZ_RAVU_ZOOM && (d->ar_strength != 0.0f) != (d->lut_ar != nullptr)) {
    delete m;
    return fail(PZ_EINVAL, "ravu-zoom anti-ringing needs the _ar LUT and a strength");
  }
  m->lut_rows = d->lut_rows;
  m->lut_cols = d->lut_cols;
  const size_t nval = (size_t)d->lut_rows * d->lut_cols * 4, bytes = nval * 4;
  auto rounded = [&](const float* src) {  // every value rounded to FP16 (round to nearest even)
    std::vector<float> r(nval);
    for (size_t i = 0; i < nval; i++) r[i] = __half2float(__float2half_rn(src[i]));
    return r;
  };
  // FP16 texels of the fast form, each row padded to an even texel count so
  // that texel pairs are 16-byte loads
  m->lut_h_pitch = (d->lut_cols + 1) & ~1;
  std::vector<__half> luth((size_t)d->lut_rows * m->lut_h_pitch * 4, __float2half_rn(0.0f));
  for (int r = 0; r < d->lut_rows; r++)
    for (int c = 0; c < d->lut_cols * 4; c++)
      luth[(size_t)r * m->lut_h_pitch * 4 + c] = __float2half_rn(d->lut[(size_t)r * d->lut_cols * 4 + c]);
  const std::vector<float> lut16 = rounded(d->lut);
  if ((rc = upload(&m->d_lut, d->lut, bytes)) || (rc = upload(&m->d_lut16, lut16.data(), bytes)) ||
      (rc = upload(&m->d_lut_h, luth.data(), luth.size() * 2))) {
    pz_model_destroy(m);
    return rc;
  }
  if (d->lut_ar) {
    const std::vector<float> ar16 = rounded(d->lut_ar);
    if ((rc = upload(&m->d_lut_ar, d->lut_ar, bytes)) || (rc = upload(&m->d_lut_ar16, ar16.data(), bytes))) {
      pz_model_destroy(m);
      return rc;
    }
  }
  *out = m;
  return PZ_OK;
}

void pz_model_destroy(pz_model* m) {
  if (!m) return;
  cudaFree(m->d_lut);
  cudaFree(m->d_lut_ar);
  cudaFree(m->d_lut16);
  cudaFree(m->d_lut_ar16);
  cudaFree(m->d_lut_h);
  cudaFree(m->d_wts);
  cudaFree(m->d_cs);
  cudaFree(m->d_bias);
  cudaFree(m->d_wts_h);
  delete m;
}

static int nn_axes(const pz_opts* o) {
  int ax = o ? o->nnedi3_axes : 0;
  return ax == 0 ? 3 : ax;
}

int pz_query(const pz_model* m, int in_w, int in_h, int dtype, const pz_opts* o, pz_query_result* r) {
  if (!m || !r) return fail(PZ_EINVAL, "null argument");
  if (in_w <= 0 || in_h <= 0) return fail(PZ_EINVAL, "bad input size %dx%d", in_w, in_h);
  if (dtype != PZ_F32 && dtype != PZ_F16) return fail(PZ_EINVAL, "unknown dtype %d", dtype);
  r->family = m->family;
  r->n_planes = m->channels == PZ_LUMA ? 1 : 3;
  r->scratch_bytes = 0;
  switch (m->family) {
    case PZ_RAVU_3X:
      r->out_width = 3 * in_w;
      r->out_height = 3 * in_h;
      break;
    case PZ_RAVU_ZOOM:
      if (!o || o->out_width <= in_w || o->out_height <= in_h)
        return fail(PZ_EINVAL, "ravu-zoom needs opts->out_width/out_height above the input size");
      r->out_width = o->out_width;
      r->out_height = o->out_height;
      break;
    case PZ_NNEDI3: {
      const int ax = nn_axes(o);
      r->out_width = (ax & 2) ? 2 * in_w : in_w;
      r->out_height = (ax & 1) ? 2 * in_h : in_h;
      if (ax == 3) r->scratch_bytes = (size_t)2 * in_h * in_w * dtype_size(dtype);
      break;
    }
    default:
      r->out_width = 2 * in_w;
      r->out_height = 2 * in_h;
      if (m->family == PZ_RAVU) r->scratch_bytes = pz::lattice_scratch_bytes(m, in_w, in_h);
  }
  return PZ_OK;
}

size_t pz_scratch_bytes(const pz_model* m, const pz_plane* in, const pz_opts* o) {
  if (!m || !in) return 0;
  if (m->family == PZ_RAVU) return pz::lattice_scratch_bytes(m, in->width, in->height);
  if (m->family != PZ_NNEDI3 || nn_axes(o) != 3) return 0;
  return (size_t)2 * in->height * in->width * dtype_size(in->dtype);
}

int pz_run(const pz_model* m, const pz_plane* in, int n_in, pz_plane* out, int n_out, const pz_opts* o,
           void* stream) {
  if (!m || !in || !out) return fail(PZ_EINVAL, "null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int C = m->channels == PZ_LUMA ? 1 : 3;
  if (n_in != C || n_out != C) return fail(PZ_EINVAL, "model needs %d planes, got %d in / %d out", C, n_in, n_out);
  int rc;
  const bool pairs = m->family == PZ_RAVU_LITE || m->family == PZ_RAVU || (m->family == PZ_NNEDI3 && (nn_axes(o) & 2));
  for (int c = 0; c < C; c++) {
    if ((rc = check_plane(in[c], "in", c, false)) || (rc = check_plane(out[c], "out", c, pairs))) return rc;
    if (in[c].width != in[0].width || in[c].height != in[0].height)
      return fail(PZ_EINVAL, "input planes differ in size");
    if (in[c].dtype != in[0].dtype || out[c].dtype != in[0].dtype)
      return fail(PZ_EINVAL, "all planes must share one dtype");
    if (out[c].width != out[0].width || out[c].height != out[0].height)
      return fail(PZ_EINVAL, "output planes differ in size");
  }
  const int W = in[0].width, H = in[0].height, dt = in[0].dtype;
  if ((rc = pz::check_opts(o, dt))) return rc;
  int* err = pz::device_error_word();
  if (!err) return fail(PZ_EIO, "device error word: cudaGetSymbolAddress failed");
  int OW = 2 * W, OH = 2 * H;
  if (m->family == PZ_RAVU_3X) {
    OW = 3 * W;
    OH = 3 * H;
  } else if (m->family == PZ_RAVU_ZOOM) {
    if (!o) return fail(PZ_EINVAL, "ravu-zoom needs opts->out_width/out_height");
    OW = o->out_width;
    OH = o->out_height;
    if (OW <= W || OH <= H)
      return fail(PZ_EINVAL, "ravu-zoom upscales only (//!WHEN in < out): %dx%d -> %dx%d", W, H, OW, OH);
  } else if (m->family == PZ_NNEDI3) {
    const int ax = nn_axes(o);
    OW = (ax & 2) ? 2 * W : W;
    OH = (ax & 1) ? 2 * H : H;
  }
  if (out[0].width != OW || out[0].height != OH)
    return fail(PZ_EINVAL, "output must be %dx%d, got %dx%d", OW, OH, out[0].width, out[0].height);

  if (m->family == PZ_NNEDI3) {
    const int ax = nn_axes(o);
    const bool fast = o && o->precision == PZ_PREC_FAST && pz::nnedi3_tc_supported(m->nns, m->win_h);
    pz::NnArgs a{};
    a.nns = m->nns;
    a.win_h = m->win_h;
    a.wts = m->d_wts;
    a.cs = m->d_cs;
    a.bias = m->d_bias;
    a.wts_h = m->d_wts_h;
    a.err = err;
    void* tmp = nullptr;
    bool own_tmp = false;
    if (ax == 3) {
      const size_t need = (size_t)2 * H * W * dtype_size(dt);
      if (o && o->scratch) {
        if (o->scratch_bytes < need) return fail(PZ_EINVAL, "scratch %zu bytes < %zu needed", o->scratch_bytes, need);
        tmp = o->scratch;
      } else {
        cudaError_t e = cudaMallocAsync(&tmp, need, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(scratch)");
        own_tmp = true;
      }
    }
    auto pass = [&](bool xpass, const void* src, int sw, int sh, int spitch, void* dst, int dpitch) {
      a.in = src;
      a.in_pitch = spitch;
      a.out = dst;
      a.out_pitch = dpitch;
      a.W = sw;
      a.H = sh;
      return fast ? pz::launch_nnedi3_tc(a, xpass, dt, s) : pz::launch_nnedi3_simt(a, xpass, dt, s);
    };
    rc = 0;
    if (ax == 3) {
      rc = pass(false, in[0].data, W, H, in[0].pitch, tmp, W);
      if (!rc) rc = pass(true, tmp, W, 2 * H, W, out[0].data, out[0].pitch);
    } else if (ax == 1) {
      rc = pass(false, in[0].data, W, H, in[0].pitch, out[0].data, out[0].pitch);
    } else {
      rc = pass(true, in[0].data, W, H, in[0].pitch, out[0].data, out[0].pitch);
    }
    if (own_tmp) cudaFreeAsync(tmp, s);
    if (rc) return fail(rc, "NNEDI3 launch configuration not supported");
  } else {
    pz::RavuArgs a{};
    for (int c = 0; c < C; c++) {
      a.in[c] = in[c].data;
      a.in_pitch[c] = in[c].pitch;
      a.out[c] = out[c].data;
      a.out_pitch[c] = out[c].pitch;
    }
    a.W = W;
    a.H = H;
    a.OW = OW;
    a.OH = OH;
    pz::select_lut(m, o ? o->precision : PZ_PREC_FP32, &a);
    a.ar = m->ar;
    a.keys = o ? o->keys : nullptr;
    a.err = err;
    a.staging = o ? o->staging : 0;
    a.tile_rows = o && o->tile_rows ? o->tile_rows : pz::default_tile_rows(m);
    a.kp = m->kp;
    bool own_i11 = false;
    if (m->family == PZ_RAVU) {  // the int11 plane between the two lattice launches
      const size_t need = pz::lattice_scratch_bytes(m, W, H);
      if (o && o->scratch) {
        if (o->scratch_bytes < need) return fail(PZ_EINVAL, "scratch %zu bytes < %zu needed", o->scratch_bytes, need);
        if (reinterpret_cast<uintptr_t>(o->scratch) % 4) return fail(PZ_EINVAL, "scratch not 4-byte aligned");
        a.i11 = static_cast<float*>(o->scratch);
      } else {
        void* tmp = nullptr;
        cudaError_t e = cudaMallocAsync(&tmp, need, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(scratch)");
        a.i11 = static_cast<float*>(tmp);
        own_i11 = true;
      }
    }
    switch (m->family) {
      case PZ_RAVU_LITE: rc = pz::launch_lite(a, m->radius, m->ar != 0.0f, dt, s); break;
      case PZ_RAVU_3X: rc = pz::launch_3x(a, m->radius, m->channels, dt, s); break;
      case PZ_RAVU: rc = pz::launch_lattice(a, m->radius, m->channels, dt, s); break;
      case PZ_RAVU_ZOOM: rc = pz::launch_zoom(a, m->radius, m->channels, m->ar != 0.0f, dt, s); break;
      default: rc = PZ_EINVAL;
    }
    if (own_i11) cudaFreeAsync(a.i11, s);
    if (rc) return fail(rc, "no kernel for family %d radius %d", m->family, m->radius);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  return PZ_OK;
}

int pz_check_device_error(void* cuda_stream) {
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  int* w = pz::device_error_word();
  if (!w) return fail(PZ_EIO, "device error word: cudaGetSymbolAddress failed");
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  int code = 0;
  e = cudaMemcpy(&code, w, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the device error word");
  if (code == pz::kErrNone) return PZ_OK;
  const int zero = 0;
  e = cudaMemcpy(w, &zero, sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "clearing the device error word");
  switch (code) {
    case pz::kErrWaitTimeout:
      return fail(PZ_ETIMEDOUT, "a bounded device-side wait ran out; the tiles of that launch were not written");
    case pz::kErrTileOverflow:
      return fail(PZ_EIO, "a ravu-zoom tile needed more input than its staging area (downscale?)");
    default:
      return fail(PZ_EIO, "device error code %d", code);
  }
}

int pz_selftest_wait(long long limit_ns, void* cuda_stream) {
  if (limit_ns < 0) return fail(PZ_EINVAL, "negative wait limit");
  int* w = pz::device_error_word();
  if (!w) return fail(PZ_EIO, "device error word: cudaGetSymbolAddress failed");
  wait_selftest_kernel<<<1, 32, 0, static_cast<cudaStream_t>(cuda_stream)>>>(w, (unsigned long long)limit_ns);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  return PZ_OK;
}

}  // extern "C"
