/*
 * pyvr_gb300 -- C ABI of the GB300 (sm_103a) volume ray marcher.
 *
 * Replaces the GL path behind pyvr's VolumeRenderer
 * (pyvr/moderngl_renderer/renderer.py + manager.py + pyvr/shaders/volume.*.glsl).
 * Plain C types only: host pointers, device pointers as void*, sizes as ints,
 * a CUDA stream as void* (NULL = the renderer's own stream).
 *
 * Every function returns PVR_OK (0) or an error code; pvr_last_error()
 * gives the message of the calling thread's most recent error.  The Python
 * shim maps PVR_ERR_VALUE -> ValueError, PVR_ERR_TYPE -> TypeError,
 * PVR_ERR_STATE / PVR_ERR_CUDA -> RuntimeError, PVR_ERR_NOMEM -> MemoryError,
 * following the reference's conventions (renderer.py:77-87, 122-127;
 * manager.py:87-88, 120-121, 190-225).
 *
 * Threading: a handle is driven by one thread at a time (like the single GL
 * context of manager.py:26); different handles may be used concurrently.
 */
#ifndef PYVR_GB300_H
#define PYVR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PVR_ABI_VERSION 1

enum pvr_status {
    PVR_OK = 0,
    PVR_ERR_VALUE = 1,       /* bad argument value (ValueError)            */
    PVR_ERR_TYPE = 2,        /* unsupported dtype / kind (TypeError)       */
    PVR_ERR_STATE = 3,       /* call order / missing state (RuntimeError)  */
    PVR_ERR_CUDA = 4,        /* CUDA runtime error (RuntimeError)          */
    PVR_ERR_NOMEM = 5,       /* device allocation failed (MemoryError)     */
    PVR_ERR_TIMEOUT = 6      /* bounded wait expired (TimeoutError)        */
};

enum pvr_dtype { PVR_U8 = 0, PVR_F16 = 1, PVR_F32 = 2 };

/* normals of a volume resource */
enum pvr_normals { PVR_NORMALS_NONE = 0, PVR_NORMALS_GIVEN = 1, PVR_NORMALS_DEVICE = 2 };

typedef struct pvr_renderer pvr_renderer;
typedef struct pvr_volume pvr_volume;
typedef struct pvr_lut pvr_lut;
typedef struct pvr_batch pvr_batch;

/* Library identity and the calling thread's last error message (no
 * counterpart in the reference, which raises Python exceptions directly). */
int pvr_abi_version(void);
const char *pvr_last_error(void);

/* ModernGLManager(width, height) + shader load (manager.py:14-41, 43-75;
 * renderer.py:34-105).  Binds to the current CUDA device; creates the
 * handle's stream and its RGBA8 target.  Default state matches the
 * reference constructor: bounds +-0.5 (renderer.py:101-102), balanced config
 * (renderer.py:70-73), Light.default() (renderer.py:82-83). */
int pvr_create(int width, int height, pvr_renderer **out);

/* ModernGLManager.cleanup (manager.py:238-256): frees every device buffer. */
int pvr_destroy(pvr_renderer *r);

/* load_volume voxel part: create_volume_texture + bounds uniforms
 * (renderer.py:107-141, manager.py:77-108).  `data` is the host (D,H,W)
 * C-order array in its own storage type; it stays in that type on the device.
 * `value_scale` multiplies the interpolated stored value (1.0 reproduces the
 * reference, which samples uint8 voxels as 0..255; 1/255 reads them as
 * UNORM).  Clears any normals of the previous volume. */
int pvr_load_volume(pvr_renderer *r, const void *data, int dtype, int d, int h, int w,
                    float value_scale, const float min_bounds[3], const float max_bounds[3]);

/* load_volume normal part: create_normal_texture (manager.py:110-135).
 * `normals` is host float32 (D,H,W,3) for the loaded volume, or NULL to drop
 * them (the march then shades with normalize(density, 0, 0), which is what
 * the reference's unbound normal sampler reads, renderer.py:143-146). */
int pvr_load_normals(pvr_renderer *r, const float *normals);

/* Volume.compute_normals / compute_normal_volume on the device
 * (pyvr/volume/data.py:103-118, pyvr/datasets/synthetic.py:109-122) for the
 * loaded volume: numpy.gradient of the stored values (central inside,
 * one-sided on faces) / (|g| + 1e-8), in the arithmetic numpy uses for the
 * storage type (float64 for uint8, float16 for float16, float32 for
 * float32).  Replaces loaded normals; needs every extent >= 2. */
int pvr_compute_normals(pvr_renderer *r);

/* set_transfer_functions -> create_rgba_transfer_function_texture
 * (renderer.py:190-207, manager.py:137-186): `rgba` is host float32
 * (size, 4).  Replaces the previous table (the reference leaks one). */
int pvr_set_lut(pvr_renderer *r, const float *rgba, int size);

/* set_camera (renderer.py:148-172): the raw float32 bytes of
 * Camera.get_view_matrix() and get_projection_matrix(w/h) as numpy holds
 * them (read column-major, as GL does, manager.py:188-192) and the camera
 * position.  Both inverses are formed here in double. */
int pvr_set_camera(pvr_renderer *r, const float view[16], const float proj[16],
                   const float camera_pos[3]);

/* set_light -> _update_light (renderer.py:174-188, 311-316). */
int pvr_set_light(pvr_renderer *r, const float position[3], const float target[3],
                  float ambient, float diffuse);

/* set_config -> _update_render_config (renderer.py:229-249, 303-309). */
int pvr_set_config(pvr_renderer *r, float step_size, int max_steps, float reference_step_size);

/* render() (renderer.py:209-219): clear, march, blend, read back.
 * out_rgba8: host buffer of width*height*4 bytes, bottom row first
 * (manager.py:228-230).  out_rgba32f: optional host buffer of
 * width*height*4 floats receiving the pre-blend fragment colour.
 * Synchronous.  With no volume loaded the image is transparent black. */
int pvr_render(pvr_renderer *r, uint8_t *out_rgba8, float *out_rgba32f);

/* render() (renderer.py:209-219) into the handle's own page-locked RGBA8
 * image (width*height*4 bytes, allocated on first use): the image comes
 * back by DMA with no staging copy, and *rgba8 receives its address.  The
 * buffer stays valid, unchanged, until the next render call on the handle or
 * pvr_destroy; a binding copies it into the `bytes` it returns.  Synchronous;
 * the same image as pvr_render. */
int pvr_render_pinned(pvr_renderer *r, const uint8_t **rgba8);

/* Same march into caller-owned DEVICE buffers on `stream` (NULL = the
 * handle's stream); asynchronous, no host copy.  Either output may be NULL. */
int pvr_render_device(pvr_renderer *r, void *d_rgba8, void *d_rgba32f, void *stream);

/* Launch shape of this handle's march (see pvr_tuning below). */
struct pvr_tuning_s;
int pvr_set_tuning(pvr_renderer *r, const struct pvr_tuning_s *tuning);

/* In-box samples (loop iterations whose texture coordinate is valid,
 * volume.frag.glsl:92) counted by the most recent render on this handle;
 * waits for that render. */
int pvr_last_sample_count(pvr_renderer *r, long long *samples);

/* Both counters of the most recent render: in-box samples (as above) and the
 * samples actually fetched and shaded (in-box samples minus those skipped in
 * bricks that are transparent under the current LUT); waits for that render. */
int pvr_last_sample_counts(pvr_renderer *r, long long *inbox, long long *shaded);

/* Bytes of device memory this handle holds. */
int pvr_device_bytes(pvr_renderer *r, long long *bytes);

/* Host-only (no CUDA call): the per-frame constants the march derives from
 * the reference's uniforms (volume.frag.glsl:3-19, 26, 50-52, 101, 107):
 * out[0..7] rows 0-1 of inverse(projection), out[8..19] rows 0-2 of
 * inverse(view), out[20..22] normalize(light_target - light_position),
 * out[23..25] 1/(max_bounds - min_bounds), out[26] step/reference_step. */
int pvr_frame_constants(const float view[16], const float proj[16], const float light_pos[3],
                        const float light_target[3], const float min_bounds[3],
                        const float max_bounds[3], float step_size, float reference_step_size,
                        float out[27]);

/* ------------------------------------------------------------------------
 * Resources and batched rendering (no single reference counterpart: these
 * split ModernGLManager's per-renderer textures, manager.py:77-186, into
 * shareable device objects so many renders run in one launch).
 * ------------------------------------------------------------------------ */

/* A volume on the device: the bricked texel records the march reads (the
 * volume and normal textures of manager.py:77-135), laid out on the device
 * from the (D,H,W) voxels of `data`, which are uploaded in their own storage
 * type and released once the records (which hold every stored value) exist.  normals_mode: PVR_NORMALS_NONE (shade
 * with normalize(density,0,0)), PVR_NORMALS_GIVEN (`normals` = host float32
 * (D,H,W,3)), PVR_NORMALS_DEVICE (computed on the device with the semantics
 * of pyvr/datasets/synthetic.py:109-122 compute_normal_volume, in the
 * arithmetic numpy uses for the storage type; needs every extent >= 2).
 * brick_log2: 2, 3 or 4 (bricks of 4^3, 8^3, 16^3 texels), or 0 for the
 * default 8^3.  Synchronous. */
int pvr_volume_create(const void *data, int dtype, int d, int h, int w, float value_scale,
                      const float min_bounds[3], const float max_bounds[3], const float *normals,
                      int normals_mode, int brick_log2, pvr_volume **out);
/* As pvr_volume_create, but returns once the upload and the layout are
 * queued (on a stream of the volume's own, at the highest priority) instead
 * of when they are done: a serving loader hands the volume on at once, and
 * every render, batch and release of the volume waits on the device for its
 * layout (the server, pvr_batch_render and pvr_batch_render_static do this
 * themselves).  `data` (and `normals`) must stay valid and unchanged until
 * pvr_volume_ready reports 1.  Layouts of pvr_set_compact_records(1) keep
 * their float records here (that compaction needs the finished layout).  No
 * reference counterpart. */
int pvr_volume_create_async(const void *data, int dtype, int d, int h, int w, float value_scale,
                            const float min_bounds[3], const float max_bounds[3], const float *normals,
                            int normals_mode, int brick_log2, pvr_volume **out);
/* *ready = 1 once the volume's layout has completed (always for volumes
 * from pvr_volume_create), else 0. */
int pvr_volume_ready(const pvr_volume *v, int *ready);
int pvr_volume_destroy(pvr_volume *v);   /* waits for the whole device first */
/* Free the volume's memory in order on `stream` without waiting: the caller
 * makes `stream` wait for every batch that reads the volume.  The handle is
 * invalid on return. */
int pvr_volume_release(pvr_volume *v, void *stream);
int pvr_volume_device_bytes(const pvr_volume *v, long long *bytes);
/* Grow the memory pool that volume resources are allocated from (the
 * current device's stream-ordered pool, which keeps what is freed) to at
 * least `bytes`, so that volumes created and released later (a serving cache
 * under a byte budget) take their memory from the pool instead of mapping
 * new memory while renders run.  No reference counterpart. */
int pvr_reserve_volume_memory(long long bytes);
/* Page-locked host memory for volume data (cudaHostAlloc, portable to every
 * device), freed with pvr_host_free.  pvr_volume_create uploads from it at
 * the link's full speed; on Grace-Blackwell, uploads from pageable memory
 * registered with cudaHostRegister ran several times slower, with 10-70 ms
 * tails for 100-250 MB volumes.  *out is NULL on failure (PVR_ERR_NOMEM when
 * the memory is not available).  No reference counterpart (moderngl uploads
 * from the numpy array, manager.py:88-97). */
int pvr_host_alloc(long long bytes, void **out);
int pvr_host_free(void *p);
/* Bytes per texel record of the volume's layout: 16 (float value + float
 * normal) or 8 (the same four floats as halves, used when every one of them
 * is a half exactly -- float16 volumes with normals computed in half
 * precision, as numpy does for float16 input).  No reference counterpart:
 * the GL path keeps voxels and normals in two textures (manager.py:77-135). */
int pvr_volume_record_bytes(const pvr_volume *v, int *bytes);
/* This volume's records as halves, if every one of their floats is a half
 * exactly; *compacted (may be NULL) = 1 if the records are halves afterwards.
 * The call first waits for all work queued on the volume's device (renders
 * queued earlier may still read the records it replaces); no render of the
 * volume may be queued while the call runs.  No reference counterpart. */
int pvr_volume_compact(pvr_volume *v, int *compacted);
/* Which layouts built after the call use 8-byte half records {value, nx, ny,
 * nz} instead of 16-byte float records (no reference counterpart; the GL
 * path keeps voxels and normals in two textures, manager.py:77-135):
 * PVR_RECORDS_FLOAT (0, the default): never; PVR_RECORDS_HALF_EXACT (1): when
 * every value and normal component is a half exactly (the images are then
 * identical); PVR_RECORDS_HALF_NORMALS (2): when every value is a half
 * exactly (uint8 and float16 volumes keep their values), with the normal
 * components rounded to half (relative error <= 2^-11 each).  Half records
 * halve the records' memory and the bytes a sample reads, and cost two
 * decode instructions per record. */
enum pvr_records { PVR_RECORDS_FLOAT = 0, PVR_RECORDS_HALF_EXACT = 1, PVR_RECORDS_HALF_NORMALS = 2 };
int pvr_set_compact_records(int mode);
int pvr_get_compact_records(int *mode);
/* *exact = 1 if the volume's records hold its values and normals exactly
 * (float records, or half records of halves), 0 if normals were rounded. */
int pvr_volume_records_exact(const pvr_volume *v, int *exact);

/* Arithmetic of the march for renders queued after the call, on every
 * entry point (no reference counterpart: GLSL leaves rounding to the
 * driver).  PVR_ARITH_FAST (0, the default): the same samples of the same
 * texels with the same lerps and LUT addressing as the exact arithmetic;
 * the shading tail contracts products into FMAs and takes exp and 1/sqrt
 * from one hardware instruction each, so images are within 1 LSB per RGBA8
 * channel of the exact ones, not bit-identical.  PVR_ARITH_EXACT (1): every
 * operation rounded as the CPU oracle rounds it, so images equal the
 * oracle's bit for bit.  A call reads the setting once for all its jobs. */
enum pvr_arithmetic { PVR_ARITH_FAST = 0, PVR_ARITH_EXACT = 1 };
int pvr_set_arithmetic(int mode);
int pvr_get_arithmetic(int *mode);
/* The float32 (D,H,W,3) normals held in the records (host buffer): what
 * Volume.normals holds after compute_normal_volume (pyvr/volume/data.py:103-118),
 * read back from the device. */
int pvr_volume_read_normals(const pvr_volume *v, float *normals_out);

/* The combined RGBA table of create_rgba_transfer_function_texture
 * (manager.py:137-186) as a device object: host float32 (size, 4). */
int pvr_lut_create(const float *rgba, int size, pvr_lut **out);
int pvr_lut_update(pvr_lut *lut, const float *rgba, int size);
int pvr_lut_destroy(pvr_lut *lut);

/* Build the LUT on the device from control points (the table
 * set_transfer_functions makes on the host: ColorTransferFunction.to_lut /
 * OpacityTransferFunction.to_lut, pyvr/transferfunctions/color.py:185-197,
 * opacity.py:185-193, combined as in manager.py:162-175): entry i of each
 * channel is numpy.interp(linspace(0, 1, size)[i], x, values) in double,
 * rounded to float32.  Host arrays: ctf_x[n_ctf], ctf_rgb[n_ctf*3],
 * otf_x[n_otf], otf_a[n_otf]; positions finite and sorted; 1..256 points per
 * function; size 1..65536.  Queued on `stream` (no host synchronisation
 * unless the table grows); no batch reading this LUT may be in flight. */
int pvr_lut_build(pvr_lut *lut, const double *ctf_x, const double *ctf_rgb, int n_ctf,
                  const double *otf_x, const double *otf_a, int n_otf, int size, void *stream);

/* Copy the LUT (size x 4 float32) to host memory; waits for the device. */
int pvr_lut_read(const pvr_lut *lut, float *rgba_out);

/* One render of a batch: the uniforms of renderer.py:148-188, 303-316 plus
 * its resources and device output buffers. */
typedef struct {
    const pvr_volume *volume;
    const pvr_lut *lut;
    int width, height;
    float view[16], proj[16], camera_pos[3];   /* as for pvr_set_camera */
    float light_pos[3], light_target[3];
    float ambient, diffuse;
    float step_size, reference_step_size;
    int max_steps;
    void *d_rgba8;                  /* device, width*height*4 bytes, or NULL */
    void *d_rgba32f;                /* device, width*height*4 floats, or NULL */
    unsigned long long *d_counters; /* device [in-box, shaded] samples (zeroed by the caller), or NULL */
} pvr_job;

/* Launch shape of the persistent batch kernel: tile_w x tile_h pixels per
 * 256-thread block (tile_w a multiple of 8, tile_h of 4, product 256),
 * march steps per loop iteration (1 or 4), persistent blocks per SM
 * (0 = as many as fit). */
typedef struct pvr_tuning_s {
    int tile_w, tile_h, steps_per_iter, blocks_per_sm;
} pvr_tuning;

/* ---- Batches (no counterpart in the reference, which renders one frame per
 * GL draw: renderer.py:209-219) -----------------------------------------
 * A batch launcher with `slots` staging slots (batches that may be in flight
 * at once).  Each batch is one persistent kernel over a shared work queue of
 * pixel tiles, launched as a captured CUDA graph. */
int pvr_batch_create(int capacity_jobs, int slots, pvr_batch **out);
int pvr_batch_destroy(pvr_batch *b);
int pvr_batch_set_tuning(pvr_batch *b, const pvr_tuning *tuning);
int pvr_batch_get_tuning(const pvr_batch *b, pvr_tuning *tuning);
/* Queue a batch of n jobs on `stream` (NULL = the batch's stream); returns
 * once it is queued.  All jobs' volumes must share one brick size. */
int pvr_batch_render(pvr_batch *b, const pvr_job *jobs, int n, void *stream);
/* Wait for every batch queued on this launcher. */
int pvr_batch_synchronize(pvr_batch *b);

/* Batch render that allocates nothing (no counterpart in the reference,
 * which renders one frame per call): the persistent batch march of
 * pvr_batch_render without a pvr_batch launcher, for callers that may not
 * allocate or free device memory (a process whose device memory all belongs
 * to its own pool, a frame loop with a fixed budget, a host that must not add
 * the device-wide synchronisation of cudaFree).  Its scratch -- one tile
 * counter per launch of up to 96 jobs, cleared to 0 by the call on `stream`
 * -- is a static 256-byte device array, so a call takes at most 6144 jobs
 * (PVR_ERR_VALUE beyond, nothing queued).  Calls whose work may overlap on a
 * device race on that array: keep them on one stream or order them.  The
 * first call on a device looks the array up (cudaGetSymbolAddress), and so
 * does the first call after the device's context was replaced
 * (cudaDeviceReset): make those calls outside stream capture.  tuning: NULL for the default; stream: NULL for
 * the default stream. */
int pvr_batch_render_static(const pvr_job *jobs, int n, const pvr_tuning *tuning, void *stream);

/* ---- Differentiable march (no counterpart in the reference) ----------
 * Gradients of an image loss with respect to the RGBA LUT and the voxel
 * values of an FP32 volume, for several views of one scene.  Device
 * pointers throughout; the scene's `views` array is on the host. */
typedef struct {
    float view[16];        /* Camera.get_view_matrix() as float32, row-major bytes */
    float proj[16];        /* Camera.get_projection_matrix(width / height) */
    float camera_pos[3];
} pvr_diff_view;

typedef struct {
    const float *volume;   /* device (D,H,W) float32, C order */
    const float *normals;  /* device (D,H,W,3) float32, or NULL: normal = (density, 0, 0) */
    int d, h, w;
    float value_scale;
    const float *lut;      /* device (lut_size, 4) float32 RGBA, lut_size <= 2048 */
    int lut_size;
    float min_bounds[3], max_bounds[3];
    float light_pos[3], light_target[3];
    float ambient, diffuse;
    float step_size, reference_step_size;
    int max_steps;
    int width, height;
    int n_views;
    const pvr_diff_view *views;
} pvr_diff_scene;

/* Forward: d_image = n_views x H x W float RGBA (the renderer's float image,
 * bit for bit), d_steps = n_views x H x W loop iterations executed (kept for
 * the backward; no per-sample state is stored). */
int pvr_diff_forward(const pvr_diff_scene *scene, float *d_image, int *d_steps, void *stream);

/* Backward of pvr_diff_forward: given dL/dimage, ADDS dL/dLUT (lut_size x 4)
 * into d_grad_lut and dL/dvoxel (D x H x W) into d_grad_volume (either may
 * be NULL: not computed).  Transmittance is rebuilt by a reverse march over
 * each ray; normals are held constant. */
int pvr_diff_backward(const pvr_diff_scene *scene, const float *d_image, const int *d_steps,
                      const float *d_grad_image, float *d_grad_lut, float *d_grad_volume,
                      void *stream);

/* ---- Serving runtime (no counterpart in the reference) -----------------
 * Continuous batching of render requests over resident volumes and LUTs on
 * native threads: a scheduler forms batches from the queued requests
 * whenever one of `slots` launch slots (each with its own stream) is free,
 * and a completer copies finished images to the requests' host buffers and
 * publishes completion records.  per_frame = 1 serves one request at a time
 * (one slot, one job per launch, the next launch after the previous image
 * is in host memory): the per-frame baseline on the same machinery.
 * The caller keeps each request's volume, LUT and output buffer alive until
 * its completion has been polled. */
typedef struct pvr_server pvr_server;

enum pvr_camera_mode { PVR_CAMERA_MATRICES = 0, PVR_CAMERA_ORBIT = 1 };

typedef struct {
    pvr_volume *volume;
    pvr_lut *lut;
    int camera_mode;            /* PVR_CAMERA_MATRICES: view/proj/camera_pos; PVR_CAMERA_ORBIT: below */
    float view[16], proj[16], camera_pos[3];
    float target[3];            /* orbit camera, Camera.from_spherical fields */
    double azimuth, elevation, roll, distance;
    float init_pos[3], init_up[3];
    double fov, near_plane, far_plane;
    float light_pos[3], light_target[3];
    float ambient, diffuse;
    float step_size, reference_step_size;
    int max_steps;
    int width, height;
    uint8_t *out_rgba8;         /* host, width*height*4 bytes, bottom row first */
    int out_pinned;             /* 1: out_rgba8 is page-locked; the image is copied to it by DMA (the
                                   march writing it through the host mapping instead, with 32-byte
                                   rows over the chip-to-chip link, slowed concurrent uploads and
                                   renders several-fold on Grace-Blackwell) */
    void *wait_event;           /* cudaEvent_t the batch must wait for (e.g. the LUT's build), or NULL */
    unsigned long long tag;     /* echoed in the completion */
} pvr_request;

typedef struct {
    unsigned long long tag;
    int status;                 /* PVR_OK or the error of the batch */
    long long t_submit_ns, t_launch_ns, t_done_ns;   /* CLOCK_MONOTONIC */
} pvr_completion;

typedef struct {
    int max_batch;              /* requests per batch (1..4096) */
    int slots;                  /* batches in flight (1..16) */
    int per_frame;              /* 1: per-frame baseline */
    int instrument;             /* N > 0: kernel events and sample counters on every N-th batch */
    int linger_us;              /* with a batch in flight, hold a partial batch up to this long */
    pvr_tuning tuning;          /* tile_w == 0: default */
    long long batch_pixels;     /* > 0: a batch takes queued requests while their pixels sum to at
                                   most this (its first request always); 0: max_batch alone limits */
} pvr_server_config;

typedef struct {
    long long submitted, batches, jobs;
    int max_jobs;
    double kernel_ms;           /* summed batch-kernel event times of the instrumented batches */
    long long inbox_samples, shaded_samples;   /* ... their in-box / shaded samples */
    double algorithmic_bytes;   /* ... shaded samples x (8 voxel + 8 x 12 normal bytes) */
    long long queued;
    long long instrumented_batches, instrumented_jobs;
} pvr_server_stats;

int pvr_server_create(const pvr_server_config *cfg, pvr_server **out);
/* Validate and queue one request (any thread).  Orbit cameras are turned
 * into matrices here (pvr_camera_spherical). */
int pvr_server_submit(pvr_server *srv, const pvr_request *req);
/* Up to `max` completions; waits up to timeout_ms for the first. */
int pvr_server_poll(pvr_server *srv, pvr_completion *out, int max, int timeout_ms, int *n_out);
/* paused = 1: launch nothing (submissions queue up); 0: resume. */
int pvr_server_pause(pvr_server *srv, int paused);
int pvr_server_get_stats(pvr_server *srv, pvr_server_stats *out);
int pvr_server_reset_stats(pvr_server *srv);
const char *pvr_server_last_error(pvr_server *srv);
/* Serves every queued request, then stops the threads and frees the slots. */
int pvr_server_destroy(pvr_server *srv);

/* Orbit camera setup on the host in double precision: Camera.from_spherical
 * + get_camera_vectors / get_view_matrix / get_projection_matrix(aspect)
 * (pyvr/camera/control.py:238-351, pyvr/camera/camera.py:292-369), giving the
 * float32 view, projection and position pvr_set_camera / pvr_job take.
 * Agrees with the reference's float32 arrays to float32 rounding.  Fails
 * with PVR_ERR_VALUE (nothing written) when the rotated up vector is parallel
 * to the view direction, where the reference's basis is rounding noise. */
int pvr_camera_spherical(const float target[3], double azimuth, double elevation, double roll,
                         double distance, const float init_pos[3], const float init_up[3], double fov,
                         double near_plane, double far_plane, double aspect, float view_out[16],
                         float proj_out[16], float pos_out[3]);

#ifdef __cplusplus
}
#endif
#endif /* PYVR_GB300_H */
