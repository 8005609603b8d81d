// Device resources of the C ABI: volumes (the voxel + normal textures of
// pyvr/moderngl_renderer/manager.py:77-135 as bricked texel records) and
// RGBA LUTs (manager.py:137-186), plus the host-side derivations shared by
// the renderer and the batch launcher.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pvr_internal.h"

namespace {
thread_local std::string g_last_error;
size_t dtype_size(int dtype) { return dtype == PVR_U8 ? 1 : dtype == PVR_F16 ? 2 : 4; }
bool finite3(const float v[3]) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }
}  // namespace

namespace pvr {

int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? PVR_ERR_NOMEM : PVR_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

// Inverse of the GL matrix stored column-major in `gl`, in double, by
// Gauss-Jordan elimination with partial pivoting; inv[r*4+c].
bool invert_gl(const float gl[16], double inv[16]) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = (double)gl[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (a[piv][col] == 0.0 || std::isnan(a[piv][col])) return false;
        if (piv != col)
            for (int c = 0; c < 8; ++c) std::swap(a[piv][c], a[col][c]);
        const double p = a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] /= p;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            const double m = a[r][col];
            if (m == 0.0) continue;
            for (int c = 0; c < 8; ++c) a[r][c] -= m * a[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[r * 4 + c] = a[r][c + 4];
    return true;
}

// normalize(light_target - light_position) (volume.frag.glsl:107); 0 for a
// degenerate light, whose diffuse term the shader's max(dot(NaN,L),0) zeroes.
void light_direction(const float pos[3], const float target[3], float out[3]) {
    float l[3];
    for (int a = 0; a < 3; ++a) l[a] = target[a] - pos[a];
    const float l2 = (l[0] * l[0] + l[1] * l[1]) + l[2] * l[2];
    const float li = l2 > 0.0f ? 1.0f / std::sqrt(l2) : 0.0f;
    for (int a = 0; a < 3; ++a) out[a] = l[a] * li;
}

// Volume memory comes from the stream-ordered allocator: unlike
// cudaMalloc / cudaFree it is no synchronisation point between streams, so
// loading or evicting a volume does not stall renders running meanwhile.
// The pool keeps freed memory for reuse instead of returning it at every
// synchronisation.
// The release threshold is set once per device (the first allocation on
// each device), from any thread.
constexpr int kMaxPoolDevices = 64;
static std::atomic<bool> g_pool_configured[kMaxPoolDevices];

cudaError_t vol_alloc(void **p, size_t bytes, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < kMaxPoolDevices && !g_pool_configured[dev].load(std::memory_order_acquire)) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        g_pool_configured[dev].store(true, std::memory_order_release);
    }
    return cudaMallocAsync(p, bytes, st);
}

void vol_free(void *p, cudaStream_t st) {
    if (p) cudaFreeAsync(p, st);
}

void free_volume_buffers(pvr_volume *v, cudaStream_t st) {
    vol_free(v->d_vol, st);
    vol_free(v->d_nrm, st);
    vol_free(v->d_records, st);
    vol_free(v->d_table, st);
    vol_free(v->d_bricks, st);
    v->d_vol = v->d_nrm = nullptr;
    v->d_records = nullptr;
    v->d_table = nullptr;
    v->d_bricks = nullptr;
}

// Which layouts built from now on use 8-byte half records
// (pvr_set_compact_records): PVR_RECORDS_FLOAT never, PVR_RECORDS_HALF_EXACT
// when every value and normal component is a half exactly,
// PVR_RECORDS_HALF_NORMALS when every value is (uint8 and float16 volumes),
// normals rounded to half.
static std::atomic<int> g_compact_records{PVR_RECORDS_FLOAT};

// The arithmetic of renders queued from now on (pvr_set_arithmetic).
static std::atomic<int> g_arithmetic{PVR_ARITH_FAST};

bool arithmetic_fast() { return g_arithmetic.load(std::memory_order_relaxed) == PVR_ARITH_FAST; }

// The allocations of a volume's layout and the upload of its brick table
// (from pageable memory: on a stream with no work queued yet, the copy is
// staged and returns at once).
static int layout_prepare(pvr_volume *v, cudaStream_t st, bool &half) {
    vol_free(v->d_records, st);
    vol_free(v->d_table, st);
    vol_free(v->d_bricks, st);
    v->d_records = nullptr;
    v->d_table = nullptr;
    v->d_bricks = nullptr;
    v->records_bytes = 0;
    v->geo = make_brick_geometry(v->dims, v->log2b);
    std::vector<uint32_t> table = morton_slots(v->geo);
    const size_t nrec = (size_t)v->geo.nbricks * brick_records(v->log2b);
    // half records written directly: values of uint8 / float16 volumes are
    // halves exactly; normals are rounded to half
    half = g_compact_records.load() == PVR_RECORDS_HALF_NORMALS && v->dtype != PVR_F32;
    const size_t rec_size = half ? sizeof(uint2) : sizeof(float4);
    PVR_CUDA(vol_alloc((void **)&v->d_records, nrec * rec_size, st));
    v->records_bytes = nrec * rec_size;
    PVR_CUDA(vol_alloc((void **)&v->d_table, table.size() * sizeof(uint32_t), st));
    PVR_CUDA(vol_alloc((void **)&v->d_bricks, table.size() * sizeof(uint4), st));
    // pageable source: staged before the call returns, so `table` may go
    PVR_CUDA(cudaMemcpyAsync(v->d_table, table.data(), table.size() * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, st));
    return PVR_OK;
}

// The layout kernel over the uploaded voxels (and given normals).
static int layout_launch(pvr_volume *v, cudaStream_t st, bool half) {
    PVR_CUDA(launch_build_records(v->geo, v->dtype, v->d_vol, v->dims, v->d_nrm, v->normals_mode,
                                  v->d_table, v->d_records, half, v->d_bricks, st));
    vol_free(v->d_nrm, st);  // given normals now live in the records
    v->d_nrm = nullptr;
    v->compact = half;
    // exact when there are no normals, or when they were computed in half
    // precision (numpy's arithmetic for float16 input)
    v->compact_exact = !half || v->normals_mode == PVR_NORMALS_NONE ||
                       (v->dtype == PVR_F16 && v->normals_mode == PVR_NORMALS_DEVICE);
    return PVR_OK;
}

// Records, brick table and value ranges of a volume (once per volume).
int ensure_volume_layout(pvr_volume *v, cudaStream_t st) {
    if (v->layout_ready) return PVR_OK;
    bool half = false;
    if (int rc = layout_prepare(v, st, half)) return rc;
    if (int rc = layout_launch(v, st, half)) return rc;
    PVR_CUDA(cudaStreamSynchronize(st));  // ready for any stream
    v->layout_ready = true;
    if (g_compact_records.load() == PVR_RECORDS_HALF_EXACT) try_compact_records(v, st, false);
    return PVR_OK;
}

void volume_stream_wait(const pvr_volume *v, cudaStream_t st) {
    if (!v || !v->ready || v->ready_done.load(std::memory_order_acquire)) return;
    if (cudaEventQuery(v->ready) == cudaSuccess) {
        v->ready_done.store(true, std::memory_order_release);
        return;
    }
    cudaGetLastError();  // cudaErrorNotReady
    cudaStreamWaitEvent(st, v->ready, 0);
}

// Half records when every value and normal is a half exactly: float16
// volumes with normals computed in half precision (numpy's arithmetic for
// float16 input) always are, uint8 values are too.  The march reads half as
// many bytes per sample and decodes the same floats.  round_normals: the
// values must still be halves exactly, the normal components are rounded to
// half (relative error <= 2^-11 per component).  The float records stay when
// a float that must be exact is not a half, or when the memory for the copy
// is missing.  Nothing may read the volume meanwhile.  Returns 1 if the
// records are halves.
int try_compact_records(pvr_volume *v, cudaStream_t st, bool round_normals) {
    if (v->compact) return 1;
    const size_t nrec = v->records_bytes / sizeof(float4);
    uint2 *compact = nullptr;
    int *d_flag = nullptr;
    int inexact = 1;
    if (vol_alloc((void **)&compact, nrec * sizeof(uint2), st) == cudaSuccess) {
        if (vol_alloc((void **)&d_flag, sizeof(int), st) == cudaSuccess &&
            cudaMemsetAsync(d_flag, 0, sizeof(int), st) == cudaSuccess &&
            launch_compact_records((const float4 *)v->d_records, compact, (long long)nrec, d_flag, st) ==
                cudaSuccess)
            cudaMemcpyAsync(&inexact, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    cudaGetLastError();  // a failed allocation or launch above only means: keep the float records
    cudaStreamSynchronize(st);
    vol_free(d_flag, st);
    const int forbidden = round_normals ? 1 : 3;  // inexact values (bit 0), normals (bit 1)
    if (compact && (inexact & forbidden) == 0) {
        vol_free(v->d_records, st);
        v->d_records = compact;
        v->records_bytes = nrec * sizeof(uint2);
        v->compact = true;
        v->compact_exact = inexact == 0;
    } else {
        vol_free(compact, st);
    }
    cudaStreamSynchronize(st);
    return v->compact ? 1 : 0;
}

// Validated job -> the descriptor the kernel reads (everything the fragment
// shader derives per fragment but that is constant over the frame).
int fill_job(const pvr_job &j, int tile_w, int tile_h, bool fast, JobDesc &out) {
    std::memset(&out, 0, sizeof(out));
    if (!j.volume || !j.lut) return fail(PVR_ERR_VALUE, "job without volume or LUT");
    if (!j.volume->layout_ready) return fail(PVR_ERR_STATE, "volume layout not built");
    if (j.width <= 0 || j.height <= 0 || j.width > 32768 || j.height > 32768)
        return fail(PVR_ERR_VALUE, "job size must be in 1..32768, got %dx%d", j.width, j.height);
    if (!(j.step_size > 0.0f) || !std::isfinite(j.step_size) || !(j.reference_step_size > 0.0f) ||
        !std::isfinite(j.reference_step_size) || j.max_steps < 1)
        return fail(PVR_ERR_VALUE, "invalid step_size / reference_step_size / max_steps");
    const pvr_volume &v = *j.volume;
    MarchFrame &f = out.f;
    double ip[16], iv[16];
    if (!invert_gl(j.proj, ip)) return fail(PVR_ERR_VALUE, "projection matrix is singular");
    if (!invert_gl(j.view, iv)) return fail(PVR_ERR_VALUE, "view matrix is singular");
    for (int i = 0; i < 8; ++i) f.ip[i] = (float)ip[i];
    for (int i = 0; i < 12; ++i) f.iv[i] = (float)iv[i];
    f.width = j.width;
    f.height = j.height;
    for (int a = 0; a < 3; ++a) {
        f.cam[a] = j.camera_pos[a];
        f.bmin[a] = v.bmin[a];
        f.bmax[a] = v.bmax[a];
        f.inv_ext[a] = 1.0f / (v.bmax[a] - v.bmin[a]);
        // world x <-> texture r (extent W), y <-> t (H), z <-> s (D)
        f.ext[a] = v.geo.ext[a];
        f.fext[a] = (float)v.geo.ext[a];
        f.nb[a] = v.geo.nb[a];
    }
    f.step = j.step_size;
    f.alpha_k = j.step_size / j.reference_step_size;
    f.max_steps = j.max_steps;
    light_direction(j.light_pos, j.light_target, f.light_dir);
    f.ambient = j.ambient;
    f.diffuse = j.diffuse;
    f.value_scale = v.value_scale;
    f.lut_size = j.lut->size;
    f.flut_size = (float)j.lut->size;
    f.flut_max = (float)(j.lut->size - 1);
    f.alpha_k2 = (float)((double)f.alpha_k * 1.4426950408889634);  // * log2(e)
    out.fast = fast ? 1 : 0;
    out.records = v.d_records;
    out.compact = v.compact ? 1 : 0;
    out.bricks = v.d_bricks;
    out.lut = j.lut->d_lut;
    out.prefix = j.lut->d_prefix;
    out.out8 = (uint32_t *)j.d_rgba8;
    out.outf = (float4 *)j.d_rgba32f;
    out.counters = j.d_counters;
    out.tiles_x = (j.width + tile_w - 1) / tile_w;
    out.tiles_y = (j.height + tile_h - 1) / tile_h;
    out.normals = v.normals_mode != PVR_NORMALS_NONE;
    out.skip = j.lut->has_clear && std::isfinite(j.ambient) && std::isfinite(j.diffuse);
    return PVR_OK;
}

}  // namespace pvr

using pvr::fail;

extern "C" {

int pvr_abi_version(void) { return PVR_ABI_VERSION; }

const char *pvr_last_error(void) { return g_last_error.c_str(); }

static int create_volume(const void *data, int dtype, int d, int h, int w, float value_scale,
                         const float min_bounds[3], const float max_bounds[3], const float *normals,
                         int normals_mode, int brick_log2, bool async, pvr_volume **out) {
    if (!out) return fail(PVR_ERR_VALUE, "out is NULL");
    *out = nullptr;
    if (!data) return fail(PVR_ERR_VALUE, "volume data is NULL");
    if (dtype != PVR_U8 && dtype != PVR_F16 && dtype != PVR_F32)
        return fail(PVR_ERR_TYPE, "unsupported volume dtype code %d", dtype);
    if (d <= 0 || h <= 0 || w <= 0) return fail(PVR_ERR_VALUE, "Volume data must be 3D with positive extents");
    if ((long long)d * h * w > (1LL << 31)) return fail(PVR_ERR_VALUE, "volume larger than 2^31 voxels");
    if (!min_bounds || !max_bounds || !finite3(min_bounds) || !finite3(max_bounds))
        return fail(PVR_ERR_VALUE, "bounds must be three finite floats each");
    for (int a = 0; a < 3; ++a)
        if (!(max_bounds[a] > min_bounds[a])) return fail(PVR_ERR_VALUE, "max_bounds must be greater than min_bounds");
    if (!std::isfinite(value_scale)) return fail(PVR_ERR_VALUE, "value_scale must be finite");
    if (normals_mode < PVR_NORMALS_NONE || normals_mode > PVR_NORMALS_DEVICE)
        return fail(PVR_ERR_VALUE, "unknown normals mode %d", normals_mode);
    if (normals_mode == PVR_NORMALS_GIVEN && !normals) return fail(PVR_ERR_VALUE, "normals are NULL");
    if (normals_mode == PVR_NORMALS_DEVICE && (d < 2 || h < 2 || w < 2))
        return fail(PVR_ERR_VALUE, "Shape of array too small to calculate a numerical gradient, "
                                   "at least (edge_order + 1) elements are required.");
    if (brick_log2 == 0) brick_log2 = pvr::kDefaultBrickLog2;
    if (brick_log2 < pvr::kMinBrickLog2 || brick_log2 > pvr::kMaxBrickLog2)
        return fail(PVR_ERR_VALUE, "brick_log2 must be 2, 3 or 4");
    pvr_volume *v = new pvr_volume();
    cudaGetDevice(&v->device);
    v->dtype = dtype;
    v->dims[0] = d;
    v->dims[1] = h;
    v->dims[2] = w;
    v->value_scale = value_scale;
    v->normals_mode = normals_mode;
    v->log2b = brick_log2;
    for (int a = 0; a < 3; ++a) {
        v->bmin[a] = min_bounds[a];
        v->bmax[a] = max_bounds[a];
    }
    const size_t nvox = (size_t)d * h * w;
    // a stream of its own at the highest priority: a load holds the renders
    // queued meanwhile back by the layout's few milliseconds, while at the
    // lowest priority it waited behind render launches for tens of
    // milliseconds, and with it every request for the new volume
    cudaStream_t st = nullptr;
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    cudaError_t e = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio_high);
    if (e != cudaSuccess) {
        delete v;
        return pvr::cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    auto bail = [&](int rc) {
        cudaStreamSynchronize(st);
        pvr::free_volume_buffers(v, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        if (v->ready) cudaEventDestroy(v->ready);
        delete v;
        return rc;
    };
    // the brick table first, while the stream is empty (its pageable copy
    // then returns at once), then the voxels in their storage type
    bool half = false;
    if (int rc = pvr::layout_prepare(v, st, half)) return bail(rc);
    e = pvr::vol_alloc(&v->d_vol, nvox * dtype_size(dtype), st);
    if (e != cudaSuccess) return bail(pvr::cuda_fail(e, "allocate volume"));
    v->vol_bytes = nvox * dtype_size(dtype);
    e = cudaMemcpyAsync(v->d_vol, data, v->vol_bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return bail(pvr::cuda_fail(e, "upload volume"));
    if (normals_mode == PVR_NORMALS_GIVEN) {
        e = pvr::vol_alloc((void **)&v->d_nrm, nvox * 3 * sizeof(float), st);
        if (e != cudaSuccess) return bail(pvr::cuda_fail(e, "allocate normals"));
        e = cudaMemcpyAsync(v->d_nrm, normals, nvox * 3 * sizeof(float), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return bail(pvr::cuda_fail(e, "upload normals"));
    }
    if (int rc = pvr::layout_launch(v, st, half)) return bail(rc);
    // the records hold every stored value: the uploaded voxels are not needed
    // again (a volume resource is never laid out twice)
    pvr::vol_free(v->d_vol, st);
    v->d_vol = nullptr;
    v->vol_bytes = 0;
    e = cudaEventCreateWithFlags(&v->ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(v->ready, st);
    if (e != cudaSuccess) return bail(pvr::cuda_fail(e, "record the layout's event"));
    v->layout_ready = true;  // queued: device work on the volume waits for `ready`
    if (!async) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return bail(pvr::cuda_fail(e, "volume layout"));
        v->ready_done.store(true);
        if (pvr::g_compact_records.load() == PVR_RECORDS_HALF_EXACT) pvr::try_compact_records(v, st, false);
    }
    cudaStreamDestroy(st);  // its queued work still runs
    *out = v;
    return PVR_OK;
}

int pvr_volume_create(const void *data, int dtype, int d, int h, int w, float value_scale,
                      const float min_bounds[3], const float max_bounds[3], const float *normals,
                      int normals_mode, int brick_log2, pvr_volume **out) {
    return create_volume(data, dtype, d, h, w, value_scale, min_bounds, max_bounds, normals, normals_mode,
                         brick_log2, false, out);
}

int pvr_volume_create_async(const void *data, int dtype, int d, int h, int w, float value_scale,
                            const float min_bounds[3], const float max_bounds[3], const float *normals,
                            int normals_mode, int brick_log2, pvr_volume **out) {
    return create_volume(data, dtype, d, h, w, value_scale, min_bounds, max_bounds, normals, normals_mode,
                         brick_log2, true, out);
}

int pvr_volume_ready(const pvr_volume *v, int *ready) {
    if (!v || !ready) return fail(PVR_ERR_VALUE, "NULL argument");
    *ready = 1;
    if (!v->ready || v->ready_done.load()) return PVR_OK;
    const cudaError_t e = cudaEventQuery(v->ready);
    if (e == cudaSuccess) {
        v->ready_done.store(true);
        return PVR_OK;
    }
    if (e == cudaErrorNotReady) {
        cudaGetLastError();
        *ready = 0;
        return PVR_OK;
    }
    return pvr::cuda_fail(e, "volume layout");
}

int pvr_volume_destroy(pvr_volume *v) {
    if (!v) return PVR_OK;
    cudaDeviceSynchronize();  // no batch may still read it
    pvr::free_volume_buffers(v, 0);
    cudaDeviceSynchronize();
    if (v->ready) cudaEventDestroy(v->ready);
    delete v;
    return PVR_OK;
}

int pvr_volume_release(pvr_volume *v, void *stream) {
    if (!v) return PVR_OK;
    // behind the layout too, when it may still be running
    pvr::volume_stream_wait(v, (cudaStream_t)stream);
    pvr::free_volume_buffers(v, (cudaStream_t)stream);
    if (v->ready) cudaEventDestroy(v->ready);  // released once it has completed
    delete v;
    return PVR_OK;
}

int pvr_reserve_volume_memory(long long bytes) {
    if (bytes < 0) return fail(PVR_ERR_VALUE, "bytes must be >= 0");
    if (bytes == 0) return PVR_OK;
    cudaStream_t st = nullptr;
    PVR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    void *p = nullptr;
    cudaError_t e = pvr::vol_alloc(&p, (size_t)bytes, st);
    if (e == cudaSuccess) cudaFreeAsync(p, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return pvr::cuda_fail(e, "reserve volume memory");
    if (e2 != cudaSuccess) return pvr::cuda_fail(e2, "reserve volume memory");
    return PVR_OK;
}

int pvr_host_alloc(long long bytes, void **out) {
    if (!out) return fail(PVR_ERR_VALUE, "NULL argument");
    *out = nullptr;
    if (bytes <= 0) return fail(PVR_ERR_VALUE, "bytes must be > 0");
    cudaError_t e = cudaHostAlloc(out, (size_t)bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *out = nullptr;
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            return fail(PVR_ERR_NOMEM, "no page-locked host memory for %lld bytes", bytes);
        }
        return pvr::cuda_fail(e, "cudaHostAlloc");
    }
    return PVR_OK;
}

int pvr_host_free(void *p) {
    if (!p) return PVR_OK;
    PVR_CUDA(cudaFreeHost(p));
    return PVR_OK;
}

int pvr_set_compact_records(int mode) {
    if (mode < PVR_RECORDS_FLOAT || mode > PVR_RECORDS_HALF_NORMALS)
        return fail(PVR_ERR_VALUE, "record mode must be 0 (float), 1 (half where exact) or 2 (half normals)");
    pvr::g_compact_records.store(mode);
    return PVR_OK;
}

int pvr_get_compact_records(int *mode) {
    if (!mode) return fail(PVR_ERR_VALUE, "NULL argument");
    *mode = pvr::g_compact_records.load();
    return PVR_OK;
}

int pvr_set_arithmetic(int mode) {
    if (mode != PVR_ARITH_FAST && mode != PVR_ARITH_EXACT)
        return fail(PVR_ERR_VALUE, "arithmetic must be 0 (fast) or 1 (exact)");
    pvr::g_arithmetic.store(mode);
    return PVR_OK;
}

int pvr_get_arithmetic(int *mode) {
    if (!mode) return fail(PVR_ERR_VALUE, "NULL argument");
    *mode = pvr::g_arithmetic.load();
    return PVR_OK;
}

int pvr_volume_compact(pvr_volume *v, int *compacted) {
    if (!v) return fail(PVR_ERR_VALUE, "NULL argument");
    if (!v->layout_ready) return fail(PVR_ERR_STATE, "volume layout not built");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != v->device) cudaSetDevice(v->device);
    // Renders queued earlier on any stream may still read the float records
    // that the swap frees: wait for all work on the volume's device first.
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        if (dev != v->device) cudaSetDevice(dev);
        return pvr::cuda_fail(e, "cudaDeviceSynchronize");
    }
    cudaStream_t st = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        if (dev != v->device) cudaSetDevice(dev);
        return pvr::cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    const int c = pvr::try_compact_records(v, st, false);
    cudaStreamDestroy(st);
    if (dev != v->device) cudaSetDevice(dev);
    if (compacted) *compacted = c;
    return PVR_OK;
}

int pvr_volume_record_bytes(const pvr_volume *v, int *bytes) {
    if (!v || !bytes) return fail(PVR_ERR_VALUE, "NULL argument");
    if (!v->layout_ready) return fail(PVR_ERR_STATE, "volume layout not built");
    *bytes = v->compact ? (int)sizeof(uint2) : (int)sizeof(float4);
    return PVR_OK;
}

int pvr_volume_records_exact(const pvr_volume *v, int *exact) {
    if (!v || !exact) return fail(PVR_ERR_VALUE, "NULL argument");
    if (!v->layout_ready) return fail(PVR_ERR_STATE, "volume layout not built");
    *exact = (!v->compact || v->compact_exact) ? 1 : 0;
    return PVR_OK;
}

int pvr_volume_device_bytes(const pvr_volume *v, long long *bytes) {
    if (!v || !bytes) return fail(PVR_ERR_VALUE, "NULL argument");
    *bytes = (long long)(v->vol_bytes + v->records_bytes +
                         (size_t)v->geo.nbricks * (sizeof(uint32_t) + sizeof(uint4)));
    return PVR_OK;
}

int pvr_volume_read_normals(const pvr_volume *v, float *normals_out) {
    if (!v || !normals_out) return fail(PVR_ERR_VALUE, "NULL argument");
    if (!v->layout_ready) return fail(PVR_ERR_STATE, "volume layout not built");
    if (v->ready) PVR_CUDA(cudaEventSynchronize(v->ready));
    const size_t n = (size_t)v->dims[0] * v->dims[1] * v->dims[2] * 3;
    float *d = nullptr;
    PVR_CUDA(cudaMalloc(&d, n * sizeof(float)));
    cudaError_t e = pvr::launch_read_normals(v->geo, v->dims, v->d_table, v->d_records, v->compact, d, 0);
    if (e == cudaSuccess) e = cudaMemcpy(normals_out, d, n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return pvr::cuda_fail(e, "read normals");
    return PVR_OK;
}

int pvr_lut_create(const float *rgba, int size, pvr_lut **out) {
    if (!out) return fail(PVR_ERR_VALUE, "out is NULL");
    *out = nullptr;
    pvr_lut *l = new pvr_lut();
    cudaGetDevice(&l->device);
    int rc = pvr_lut_update(l, rgba, size);
    if (rc != PVR_OK) {
        pvr_lut_destroy(l);
        return rc;
    }
    *out = l;
    return PVR_OK;
}

int pvr_lut_update(pvr_lut *l, const float *rgba, int size) {
    if (!l) return fail(PVR_ERR_VALUE, "null LUT handle");
    if (!rgba) return fail(PVR_ERR_VALUE, "LUT is NULL");
    if (size <= 0 || size > (1 << 24)) return fail(PVR_ERR_VALUE, "LUT size must be in 1..2^24, got %d", size);
    if (size > l->cap) {
        if (l->d_lut || l->d_prefix) {
            cudaDeviceSynchronize();  // a queued batch may still read the old table
            cudaFree(l->d_lut);
            cudaFree(l->d_prefix);
            l->d_lut = nullptr;
            l->d_prefix = nullptr;
            l->cap = 0;
        }  // a new table waits for nothing
        PVR_CUDA(cudaMalloc(&l->d_lut, (size_t)size * sizeof(float4)));
        PVR_CUDA(cudaMalloc(&l->d_prefix, (size_t)(size + 1) * sizeof(int)));
        l->cap = size;
    }
    // prefix[i] = entries before i that a skipped sample must not read:
    // alpha not exactly 0, or a non-finite colour
    std::vector<int> prefix(size + 1, 0);
    for (int i = 0; i < size; ++i) {
        const float *e = rgba + 4 * i;
        const bool clear = e[3] == 0.0f && std::isfinite(e[0]) && std::isfinite(e[1]) && std::isfinite(e[2]);
        prefix[i + 1] = prefix[i] + (clear ? 0 : 1);
    }
    // copies on a non-blocking stream of this thread: they neither wait for
    // nor hold up renders on other streams (the caller guarantees that no
    // queued batch still reads this LUT)
    thread_local cudaStream_t copy_stream = nullptr;
    if (!copy_stream) PVR_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
    PVR_CUDA(cudaMemcpyAsync(l->d_lut, rgba, (size_t)size * sizeof(float4), cudaMemcpyHostToDevice, copy_stream));
    PVR_CUDA(cudaMemcpyAsync(l->d_prefix, prefix.data(), (size_t)(size + 1) * sizeof(int),
                             cudaMemcpyHostToDevice, copy_stream));
    PVR_CUDA(cudaStreamSynchronize(copy_stream));
    l->size = size;
    l->has_clear = prefix[size] < size;
    return PVR_OK;
}

int pvr_lut_destroy(pvr_lut *l) {
    if (!l) return PVR_OK;
    cudaDeviceSynchronize();
    cudaFree(l->d_lut);
    cudaFree(l->d_prefix);
    delete l;
    return PVR_OK;
}

int pvr_frame_constants(const float view[16], const float proj[16], const float light_pos[3],
                        const float light_target[3], const float min_bounds[3],
                        const float max_bounds[3], float step_size, float reference_step_size,
                        float out[27]) {
    if (!view || !proj || !light_pos || !light_target || !min_bounds || !max_bounds || !out)
        return fail(PVR_ERR_VALUE, "NULL argument");
    double ip[16], iv[16];
    if (!pvr::invert_gl(proj, ip)) return fail(PVR_ERR_VALUE, "projection matrix is singular");
    if (!pvr::invert_gl(view, iv)) return fail(PVR_ERR_VALUE, "view matrix is singular");
    for (int i = 0; i < 8; ++i) out[i] = (float)ip[i];
    for (int i = 0; i < 12; ++i) out[8 + i] = (float)iv[i];
    pvr::light_direction(light_pos, light_target, out + 20);
    for (int a = 0; a < 3; ++a) out[23 + a] = 1.0f / (max_bounds[a] - min_bounds[a]);
    out[26] = step_size / reference_step_size;
    return PVR_OK;
}

}  // extern "C"
