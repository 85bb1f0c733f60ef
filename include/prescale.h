/*
 * prescale.h -- C ABI of the GB300-native RAVU / NNEDI3 prescaler library
 * (libprescale.so).
 *
 * The reference has no library boundary of its own: its "interface" is the
 * mpv user-shader hook protocol.  A host (mpv, libplacebo) parses a .hook
 * file, uploads the //!TEXTURE blocks once, and for every frame binds the
 * hooked plane and dispatches each pass.  The entry points below are what
 * such a host binds instead of the shader passes:
 *
 *   pz_model_create   replaces the one-time //!TEXTURE upload and the
 *                     per-file constants (e.g. ravu-lite-r3.hook:132-136
 *                     LUT block; nnedi3-nns16-win8x4.hook:31-49 inline
 *                     weights; ravu-lite-ar-r3.hook:181 AR strength).
 *   pz_run            replaces one full hook chain on one frame:
 *                     ravu-lite(-ar): ravu-lite-r3.hook:15-131 (2 passes),
 *                       compute/ravu-lite-ar-r3.hook:15-171 (1 pass);
 *                     ravu: ravu-r3.hook:15-437 (4 passes),
 *                       compute/ravu-r3.hook:15-430 (2 passes);
 *                     ravu-zoom(-ar): ravu-zoom-r2.hook:15-139,
 *                       compute/ravu-zoom-ar-r2-rgb.hook:15-238;
 *                     ravu-3x: compute/ravu-3x-r2.hook:15-115;
 *                     nnedi3: nnedi3-nns16-win8x4.hook:15-210 (4 passes),
 *                       compute/nnedi3-nns128-win8x6.hook:15-448 (2 passes).
 *   pz_batch_run      replaces many such dispatches (mixed files, frames of
 *                     uneven size) issued back to back by the host, as one
 *                     persistent launch.
 *
 * Conventions: all buffers are caller-owned DEVICE memory; every call is
 * asynchronous on the given CUDA stream; return codes are 0 or a negative
 * errno value, with a message for the calling thread in pz_last_error().
 * No C++ exception crosses this boundary.  A model is immutable after
 * creation and may be used from several streams at once.
 */
#ifndef PRESCALE_H
#define PRESCALE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PZ_ABI_VERSION 2

#define PZ_OK 0
#define PZ_EINVAL (-22)
#define PZ_ENOMEM (-12)
#define PZ_EIO (-5)         /* CUDA launch or runtime error */
#define PZ_ENOTSUP (-95)
#define PZ_ETIMEDOUT (-110) /* a bounded device-side wait ran out */

typedef enum {
  PZ_RAVU_LITE = 1, /* ravu-lite, ravu-lite-ar            */
  PZ_RAVU = 2,      /* ravu (lattice: int11, int10, int01) */
  PZ_RAVU_ZOOM = 3, /* ravu-zoom, ravu-zoom-ar             */
  PZ_RAVU_3X = 4,   /* ravu-3x                             */
  PZ_NNEDI3 = 5
} pz_family;

typedef enum { PZ_LUMA = 0, PZ_YUV = 1, PZ_RGB = 2 } pz_channels;
typedef enum { PZ_F32 = 0, PZ_F16 = 1 } pz_dtype;

typedef enum {
  PZ_PREC_FP32 = 0,  /* plain FP32 arithmetic everywhere                    */
  PZ_PREC_FAST = 1,  /* FP16 tensor-core NNEDI3 neurons; ravu-lite / 3x /
                        zoom read their LUTs as FP16 texels (half the L1
                        gather traffic; zoom-ar's anti-ringing LUT stays
                        FP32), all RAVU arithmetic stays FP32               */
  PZ_PREC_MPV = 2    /* what the mpv host computes, to measure the distance
                        to it: RAVU LUTs rounded to FP16 as the host uploads
                        them (//!FORMAT rgba16f, ravu-lite-r3.hook:134),
                        ravu-zoom LUT bilinear weights in 1/256 steps as the
                        texture unit forms them; FP16 planes only (the
                        host's textures are rgba16f); NNEDI3 as PZ_PREC_FP32 */
} pz_precision;

/* Everything a .hook file contributes; host arrays are copied. */
typedef struct {
  int family;              /* pz_family                                      */
  int radius;              /* RAVU radius (2, 3, 4)                          */
  int channels;            /* pz_channels                                    */
  float ar_strength;       /* anti-ringing mix strength, 0 = none            */
  /* RAVU LUT: float32 [lut_rows][lut_cols][4] exactly as in //!TEXTURE      */
  const float* lut;
  int lut_rows, lut_cols;
  const float* lut_ar;     /* ravu-zoom-ar second LUT (same shape) or NULL   */
  /* key quantisation */
  const double* grad_weights; /* Gaussian weights of the gradient points     */
  int n_grad;
  int strength_log2;       /* 0: thresholds, 1: floor(log2(l*scale+eps))    */
  float strength_thr[3];
  int n_strength_thr;      /* 2 or 3 when strength_log2 == 0                 */
  float strength_scale;    /* e.g. 2000                                      */
  int strength_max;        /* e.g. 8                                         */
  float coherence_thr[2];  /* 0.25, 0.5                                      */
  /* NNEDI3 */
  int nns, win_w, win_h;
  const float* weights_a;  /* [win_w*win_h][nns], canonical tap order        */
  const float* weights_b;
  const float* bias_a;     /* [nns] */
  const float* bias_b;
} pz_model_desc;

typedef struct pz_model pz_model;

/* One image plane in device memory (pitch in elements). */
typedef struct {
  void* data;
  int width, height;
  int pitch;
  int dtype;               /* pz_dtype */
} pz_plane;

typedef struct {
  int precision;           /* pz_precision                                   */
  int out_width;           /* ravu-zoom target size; ignored otherwise       */
  int out_height;
  int nnedi3_axes;         /* bit 0: double rows (y), bit 1: columns (x);
                              0 means both                                   */
  int32_t* keys;           /* optional device buffer receiving the raw LUT
                              key of every key evaluation (parity tests)     */
  void* scratch;           /* optional caller scratch for multi-pass chains  */
  size_t scratch_bytes;
  int staging;             /* RAVU halo staging: 0 clamped loads, 1 TMA boxes
                              for interior tiles (border tiles always use
                              clamped loads: TMA fills zeros, not the edge)  */
  int tile_rows;           /* RAVU tile height: 4, 8 or 16 rows of 32 pixels
                              (input pixels; ravu-zoom: output pixels), one
                              thread per pixel; 0: the program's measured
                              default (4 rows; ravu-lite r2 and ravu-lite-ar
                              r4: 8).  The pixels do not depend on it.  The
                              persistent batch kernels run 8-row tiles
                              whatever this says.                           */
} pz_opts;

int pz_version(void);
const char* pz_last_error(void);

/* ---- device-side errors ------------------------------------------------
 * No counterpart in the reference (a shader cannot report an error to the
 * mpv host).  Every device-side wait of the kernels (TMA copies, tensor-core
 * MMA completion) is bounded in time; a wait that runs out abandons its
 * tile and records the failure in a per-device error word instead of
 * hanging the GPU.  pz_check_device_error waits for `cuda_stream`, reads
 * and clears that word: PZ_OK, PZ_ETIMEDOUT (a bounded wait ran out; some
 * output tiles of the launches since the last check were not written) or
 * PZ_EIO (another device-side failure), with the message in
 * pz_last_error().  The word is shared by every stream on the device. */
int pz_check_device_error(void* cuda_stream);

/* Test hook for the path above: enqueues on `cuda_stream` a kernel whose one
 * CTA waits on an mbarrier that nothing arrives at (no copy, no MMA in
 * flight), giving up after limit_ns nanoseconds and recording the timeout
 * like a real kernel would; the next pz_check_device_error returns
 * PZ_ETIMEDOUT. */
int pz_selftest_wait(long long limit_ns, void* cuda_stream);

int pz_model_create(const pz_model_desc* desc, pz_model** out);
void pz_model_destroy(pz_model* model);

/* What pz_run produces for an input size, so that a host can size its
 * buffers without knowing the file: output size (2x, 3x, the zoom target or
 * the enabled NNEDI3 axes), planes per frame and the scratch bytes pz_run
 * would allocate.  Host-only: no device call. */
typedef struct {
  int out_width, out_height;
  int n_planes;            /* 1 luma, 3 yuv / rgb                            */
  int family;              /* pz_family                                      */
  size_t scratch_bytes;    /* as pz_scratch_bytes                            */
} pz_query_result;
int pz_query(const pz_model* model, int in_width, int in_height, int dtype, const pz_opts* opts,
             pz_query_result* out);

/* Device scratch bytes pz_run needs for this model/input (0 if none). */
size_t pz_scratch_bytes(const pz_model* model, const pz_plane* in, const pz_opts* opts);

/* Run the full hook chain of `model` on one frame.  n_in/n_out planes are
 * 1 (luma) or 3 (yuv/rgb, planar).  Output sizes: 2x (lite, ravu, nnedi3),
 * 3x (3x), or opts->out_width x out_height (zoom).  ravu-lite, ravu and the
 * column pass of nnedi3 write pixel pairs: their outputs' base and pitch must
 * be 2-element aligned.  Scratch (pz_scratch_bytes): nnedi3 doubling both
 * axes, the row-doubled plane (2 * W * H * element size); ravu, the FP32
 * int11 plane between its two launches (planes * W * H * 4 bytes, 4-byte
 * aligned).  When opts->scratch is NULL and scratch is needed, it is
 * allocated stream-ordered and freed. */
int pz_run(const pz_model* model, const pz_plane* in, int n_in, pz_plane* out, int n_out,
           const pz_opts* opts, void* cuda_stream);

/* ---- frames in host memory --------------------------------------------
 * For hosts that decode in software and hold frames in host memory: runs
 * the chain over n_frames frames, copying frame i in, running it and copying
 * it back while its neighbours' transfers run under its kernels (a pair of
 * copy streams owned by the library, three device slots in `work`; calls on
 * different cuda_streams take different pairs from a pool of four, so two
 * models' calls in flight together share the host link frame by frame).  Frames are
 * planar and unpadded: frame f, plane c starts at element
 * (f * n_planes + c) * height * width of host_in; host_out likewise at the
 * output size pz_query reports.  Page-locked host memory is needed for the
 * copies to overlap.  Asynchronous: `cuda_stream` completes once the last
 * frame is in host_out.  work: device memory of pz_run_host_work_bytes()
 * bytes (three frame slots; a call of n < 3 frames needs n thirds of it),
 * 256-byte aligned, not used by anything else until the stream has passed
 * this call.  The copies first wait for the work already queued on
 * cuda_stream (which may still use `work`); with PZ_HOST_WORK_IDLE in flags
 * the caller vouches that `work` is idle, and the first frame's copy starts
 * at once, so calls for several models overlap.  Replaces a host's
 * per-frame upload, hook passes and readback. */
#define PZ_HOST_WORK_IDLE 1
size_t pz_run_host_work_bytes(const pz_model* model, int width, int height, int dtype, const pz_opts* opts);
int pz_run_host(const pz_model* model, const void* host_in, void* host_out, int n_frames, int width, int height,
                int dtype, const pz_opts* opts, void* work, size_t work_bytes, int flags, void* cuda_stream);

/* ---- batched persistent execution ------------------------------------- */

typedef struct {
  const pz_model* model;
  pz_plane in[3];
  pz_plane out[3];
  int n_planes;
  pz_opts opts;
} pz_job;

/* Many frames of many models per launch (replaces the back-to-back shader
 * dispatches a multi-stream host issues).  RAVU jobs of any mix and frame
 * size run as one persistent kernel per tile program and plane dtype whose
 * CTAs pull 32x8 tiles of every job of that program from a device counter;
 * the ravu lattice passes follow as second-phase kernels (they read the
 * int11 values of the first); NNEDI3 jobs run as their own stream-ordered
 * passes.  A job whose opts.staging is 1 has its interior tiles staged by
 * TMA inside the persistent loop too (its tensor maps sit in the job table).
 * `work` is caller device memory of at least pz_batch_work_bytes(); it
 * holds the job table and the tile counters and must stay in place while
 * the plan is used.
 *
 * pz_batch_create validates the jobs and uploads the table (synchronous on
 * `cuda_stream`); pz_batch_launch only enqueues a memset and kernels, so it
 * can be captured into a CUDA graph and replayed while the jobs' buffers
 * stay in place; pz_batch_run is create + launch + destroy.  ctas_per_sm
 * caps the persistent grid (0 = as many as fit). */
typedef struct pz_batch pz_batch;
size_t pz_batch_work_bytes(const pz_job* jobs, int n_jobs);
int pz_batch_create(const pz_job* jobs, int n_jobs, void* work, size_t work_bytes,
                    int ctas_per_sm, void* cuda_stream, pz_batch** out);
int pz_batch_launch(const pz_batch* plan, void* cuda_stream);
void pz_batch_destroy(pz_batch* plan);
int pz_batch_run(const pz_job* jobs, int n_jobs, void* work, size_t work_bytes,
                 void* cuda_stream);

/* ---- NNEDI3 without any allocation ------------------------------------
 * No counterpart in the reference: there, the mpv host owns every GPU
 * buffer.  It exists for hosts that cannot allocate device memory while a
 * frame is being rendered: a render callback against a display deadline, a
 * host that hands the library a fixed memory budget up front, or a caller
 * whose own allocator must not be re-entered.
 *
 * Same contract as pz_run for an NNEDI3 model (one luma plane in, one out),
 * but the row-doubled plane between the row and column passes comes from a
 * static device array of PZ_STATIC_SCRATCH_BYTES inside the library, and the
 * call allocates nothing.  Doubling both axes needs 2 * width * height *
 * element size bytes there (a 1920x1080 FP32 frame fits); larger frames are
 * rejected with PZ_EINVAL.  Every GPU that loads the library holds the array
 * until the process exits.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress); make that call before any
 * stream capture.  All calls share the array, so calls that overlap on the
 * GPU race on it: order them on one stream or with events.  opts->precision
 * is checked as by pz_run; a device-side wait that runs out is reported by
 * pz_check_device_error. */
#define PZ_STATIC_SCRATCH_BYTES (16u * 1024u * 1024u)
int pz_nnedi3_run_static(const pz_model* model, const pz_plane* in, pz_plane* out,
                         const pz_opts* opts, void* cuda_stream);

/* ---- resampling around the hook chain ---------------------------------
 * The scaler steps a host performs around a prescaler, for callers that want
 * the picture the host would show:
 *   - the shift a pass announces with //!OFFSET (ravu-r3.hook:424
 *     "-0.5 -0.5"; nnedi3-nns16-win8x4.hook:95 "0 -0.5", :185
 *     "-0.5 0"), which mpv folds into its next scaling pass: sx = sy = 1,
 *     (ox, oy) = the accumulated offset;
 *   - chroma upsampling (--cscale) that merges subsampled planes before a
 *     NATIVE hook (compute/ravu-r2-yuv.hook:15; README.md:50-56): sx, sy =
 *     chroma/luma size ratio, ox, oy = -(chroma siting in luma px) * ratio.
 * out(x, y) = sum k(u - i) k(v - j) in(clamp(i), clamp(j)) with
 * u = sx * x + ox, v = sy * y + oy, texel centres at integers, edges
 * replicated; k = bilinear tent or Catmull-Rom cubic.  Any sizes; in and
 * out share one dtype; asynchronous on the stream. */
typedef enum { PZ_FILTER_BILINEAR = 0, PZ_FILTER_CATMULL_ROM = 1 } pz_filter;
int pz_resample(const pz_plane* in, pz_plane* out, float sx, float ox, float sy, float oy, int filter,
                void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* PRESCALE_H */
