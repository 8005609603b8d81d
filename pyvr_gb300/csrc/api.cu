// C ABI of the renderer handle: the job of pyvr's ModernGLManager
// (pyvr/moderngl_renderer/manager.py) and of the uniform plumbing of
// ModernGLVolumeRenderer (renderer.py:303-316), on CUDA device buffers.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pvr_device.cuh"
#include "pvr_internal.h"

namespace {

thread_local std::string g_last_error;

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

#define PVR_CUDA(expr)                                              \
    do {                                                            \
        cudaError_t e_ = (expr);                                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);         \
    } while (0)

struct DeviceScope {
    int prev = -1, dev;
    explicit DeviceScope(int d) : dev(d) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceScope() {
        if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    }
};

// Inverse of the GL matrix stored column-major in `gl`, in double, by
// Gauss-Jordan elimination with partial pivoting; inv[r*4+c] (double).
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
        double p = a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] /= p;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            double m = a[r][col];
            if (m == 0.0) continue;
            for (int c = 0; c < 8; ++c) a[r][c] -= m * a[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[r * 4 + c] = a[r][c + 4];
    return true;
}

size_t dtype_size(int dtype) { return dtype == PVR_U8 ? 1 : dtype == PVR_F16 ? 2 : 4; }

}  // namespace

struct pvr_renderer {
    int device = 0;
    int width = 0, height = 0;
    cudaStream_t stream = nullptr;

    // volume (create_volume_texture)
    void *d_vol = nullptr;
    size_t vol_bytes = 0;
    int dtype = PVR_F32;
    int dims[3] = {0, 0, 0};  // D, H, W
    float value_scale = 1.0f;
    bool has_volume = false;
    // normals (create_normal_texture); only held until the records are built
    float *d_nrm = nullptr;
    size_t nrm_bytes = 0;
    bool has_normals = false;

    // bricked texel records + brick table + per-brick value range (layout.cu)
    pvr::BrickGeometry geo = {};
    float4 *d_records = nullptr;
    size_t records_bytes = 0;
    uint32_t *d_table = nullptr;
    float2 *d_minmax = nullptr;
    bool layout_dirty = true;
    bool flags_dirty = true;
    int *d_prefix = nullptr;  // count of LUT entries that are not exactly transparent
    int prefix_cap = 0;
    float bmin[3] = {-0.5f, -0.5f, -0.5f}, bmax[3] = {0.5f, 0.5f, 0.5f};

    // LUT (create_rgba_transfer_function_texture)
    float4 *d_lut = nullptr;
    int lut_size = 0, lut_cap = 0;

    // camera uniforms after the double-precision inverses
    bool has_camera = false;
    float ip[8] = {}, iv[12] = {}, cam[3] = {};

    // light + config uniforms (Light.default(), RenderConfig.balanced())
    float light_pos[3] = {1.0f, 1.0f, 1.0f}, light_target[3] = {0.0f, 0.0f, 0.0f};
    float ambient = 0.2f, diffuse = 0.8f;
    float step = 0.01f, ref_step = 0.01f;
    int max_steps = 500;

    // render targets
    uint32_t *d_out8 = nullptr;
    float4 *d_outf = nullptr;
    unsigned long long *d_samples = nullptr;  // [in-box samples, shaded samples]
};

namespace {

void free_layout(pvr_renderer *r) {
    cudaFree(r->d_records);
    cudaFree(r->d_table);
    cudaFree(r->d_minmax);
    r->d_records = nullptr;
    r->d_table = nullptr;
    r->d_minmax = nullptr;
    r->records_bytes = 0;
    r->layout_dirty = true;
}

void free_all(pvr_renderer *r) {
    free_layout(r);
    cudaFree(r->d_prefix);
    r->d_prefix = nullptr;
    cudaFree(r->d_vol);
    cudaFree(r->d_nrm);
    cudaFree(r->d_lut);
    cudaFree(r->d_out8);
    cudaFree(r->d_outf);
    cudaFree(r->d_samples);
    r->d_vol = nullptr;
    r->d_nrm = nullptr;
    r->d_lut = nullptr;
    r->d_out8 = nullptr;
    r->d_outf = nullptr;
    r->d_samples = nullptr;
}

int check_handle(pvr_renderer *r) {
    if (!r) return fail(PVR_ERR_VALUE, "null renderer handle");
    return PVR_OK;
}

bool finite3(const float v[3]) {
    return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

void light_direction(const float pos[3], const float target[3], float out[3]) {
    float l[3];
    for (int a = 0; a < 3; ++a) l[a] = target[a] - pos[a];
    float l2 = (l[0] * l[0] + l[1] * l[1]) + l[2] * l[2];
    float li = l2 > 0.0f ? 1.0f / std::sqrt(l2) : 0.0f;
    for (int a = 0; a < 3; ++a) out[a] = l[a] * li;
}

// Uniform values -> kernel frame (everything the fragment shader derives
// per fragment but that is constant over the frame).
void build_frame(const pvr_renderer *r, pvr::MarchFrame &f) {
    std::memset(&f, 0, sizeof(f));
    f.width = r->width;
    f.height = r->height;
    std::memcpy(f.ip, r->ip, sizeof(f.ip));
    std::memcpy(f.iv, r->iv, sizeof(f.iv));
    for (int a = 0; a < 3; ++a) {
        f.cam[a] = r->cam[a];
        f.bmin[a] = r->bmin[a];
        f.bmax[a] = r->bmax[a];
        f.inv_ext[a] = 1.0f / (r->bmax[a] - r->bmin[a]);
    }
    // world x <-> texture r (extent W, slowest), y <-> t (H), z <-> s (D)
    for (int a = 0; a < 3; ++a) {
        f.ext[a] = r->geo.ext[a];
        f.fext[a] = (float)f.ext[a];
        f.nb[a] = r->geo.nb[a];
    }
    f.step = r->step;
    f.alpha_k = r->step / r->ref_step;
    f.max_steps = r->max_steps;
    light_direction(r->light_pos, r->light_target, f.light_dir);
    f.ambient = r->ambient;
    f.diffuse = r->diffuse;
    f.value_scale = r->value_scale;
    f.lut_size = r->lut_size;
    f.flut_size = (float)r->lut_size;
}

int ensure_targets(pvr_renderer *r, bool want_float) {
    size_t npx = (size_t)r->width * r->height;
    if (!r->d_out8) PVR_CUDA(cudaMalloc(&r->d_out8, npx * 4));
    if (want_float && !r->d_outf) PVR_CUDA(cudaMalloc(&r->d_outf, npx * 16));
    if (!r->d_samples) PVR_CUDA(cudaMalloc(&r->d_samples, 2 * sizeof(unsigned long long)));
    return PVR_OK;
}

// Records, brick table and value ranges of the loaded volume (once per
// volume), then the transparent flags for the current LUT.
int ensure_layout(pvr_renderer *r) {
    if (r->layout_dirty) {
        free_layout(r);
        r->geo = pvr::make_brick_geometry(r->dims);
        std::vector<uint32_t> table = pvr::morton_slots(r->geo);
        size_t nrec = (size_t)r->geo.nbricks * pvr::kRecordsPerBrick;
        PVR_CUDA(cudaMalloc(&r->d_records, nrec * sizeof(float4)));
        r->records_bytes = nrec * sizeof(float4);
        PVR_CUDA(cudaMalloc(&r->d_table, table.size() * sizeof(uint32_t)));
        PVR_CUDA(cudaMalloc(&r->d_minmax, table.size() * sizeof(float2)));
        PVR_CUDA(cudaMemcpyAsync(r->d_table, table.data(), table.size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, r->stream));
        PVR_CUDA(pvr::launch_build_records(r->geo, r->dtype, r->d_vol,
                                           r->has_normals ? r->d_nrm : nullptr, r->d_table,
                                           r->d_records, r->d_minmax, r->stream));
        PVR_CUDA(cudaStreamSynchronize(r->stream));  // `table` leaves scope
        cudaFree(r->d_nrm);  // the normals now live in the records
        r->d_nrm = nullptr;
        r->nrm_bytes = 0;
        r->layout_dirty = false;
        r->flags_dirty = true;
    }
    if (r->flags_dirty && r->d_prefix) {
        bool enable = std::isfinite(r->ambient) && std::isfinite(r->diffuse);
        PVR_CUDA(pvr::launch_brick_flags(r->geo, r->value_scale, r->lut_size, r->d_prefix, enable,
                                         r->d_minmax, r->d_table, r->stream));
        r->flags_dirty = false;
    }
    return PVR_OK;
}

int march_into(pvr_renderer *r, uint32_t *d8, float4 *df, cudaStream_t st) {
    PVR_CUDA(cudaMemsetAsync(r->d_samples, 0, 2 * sizeof(unsigned long long), st));
    if (!r->has_volume) {  // unbound samplers read zero: transparent image
        size_t npx = (size_t)r->width * r->height;
        if (d8) PVR_CUDA(cudaMemsetAsync(d8, 0, npx * 4, st));
        if (df) PVR_CUDA(cudaMemsetAsync(df, 0, npx * 16, st));
        return PVR_OK;
    }
    if (!r->has_camera)
        return fail(PVR_ERR_STATE, "Camera not set: call set_camera() before render()");
    if (!r->d_lut)
        return fail(PVR_ERR_STATE,
                    "Transfer functions not set: call set_transfer_functions() before render()");
    if (int rc = ensure_layout(r)) return rc;
    if (st != r->stream) {  // layout work was queued on the handle's stream
        PVR_CUDA(cudaStreamSynchronize(r->stream));
    }
    pvr::MarchFrame f;
    build_frame(r, f);
    PVR_CUDA(pvr::launch_march(f, r->d_records, r->d_table, r->has_normals, r->d_lut, d8, df,
                               r->d_samples, st));
    return PVR_OK;
}

}  // namespace

extern "C" {

int pvr_abi_version(void) { return PVR_ABI_VERSION; }

const char *pvr_last_error(void) { return g_last_error.c_str(); }

int pvr_create(int width, int height, pvr_renderer **out) {
    if (!out) return fail(PVR_ERR_VALUE, "out is NULL");
    *out = nullptr;
    if (width <= 0 || height <= 0 || width > 32768 || height > 32768)
        return fail(PVR_ERR_VALUE, "width and height must be in 1..32768, got %dx%d", width, height);
    int dev = 0;
    PVR_CUDA(cudaGetDevice(&dev));
    pvr_renderer *r = new pvr_renderer();
    r->device = dev;
    r->width = width;
    r->height = height;
    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete r;
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    int rc = ensure_targets(r, false);
    if (rc != PVR_OK) {
        free_all(r);
        cudaStreamDestroy(r->stream);
        delete r;
        return rc;
    }
    *out = r;
    return PVR_OK;
}

int pvr_destroy(pvr_renderer *r) {
    if (!r) return PVR_OK;
    DeviceScope ds(r->device);
    cudaStreamSynchronize(r->stream);
    free_all(r);
    cudaStreamDestroy(r->stream);
    delete r;
    return PVR_OK;
}

int pvr_load_volume(pvr_renderer *r, const void *data, int dtype, int d, int h, int w,
                    float value_scale, const float min_bounds[3], const float max_bounds[3]) {
    if (int rc = check_handle(r)) return rc;
    if (!data) return fail(PVR_ERR_VALUE, "volume data is NULL");
    if (dtype != PVR_U8 && dtype != PVR_F16 && dtype != PVR_F32)
        return fail(PVR_ERR_TYPE, "unsupported volume dtype code %d", dtype);
    if (d <= 0 || h <= 0 || w <= 0) return fail(PVR_ERR_VALUE, "Volume data must be 3D with positive extents");
    if (!min_bounds || !max_bounds || !finite3(min_bounds) || !finite3(max_bounds))
        return fail(PVR_ERR_VALUE, "bounds must be three finite floats each");
    for (int a = 0; a < 3; ++a)
        if (!(max_bounds[a] > min_bounds[a]))
            return fail(PVR_ERR_VALUE, "max_bounds must be greater than min_bounds");
    if (!std::isfinite(value_scale)) return fail(PVR_ERR_VALUE, "value_scale must be finite");
    DeviceScope ds(r->device);
    size_t bytes = (size_t)d * h * w * dtype_size(dtype);
    if (bytes != r->vol_bytes) {
        PVR_CUDA(cudaStreamSynchronize(r->stream));
        cudaFree(r->d_vol);
        r->d_vol = nullptr;
        r->vol_bytes = 0;
        r->has_volume = false;
        PVR_CUDA(cudaMalloc(&r->d_vol, bytes));
        r->vol_bytes = bytes;
    }
    PVR_CUDA(cudaMemcpyAsync(r->d_vol, data, bytes, cudaMemcpyHostToDevice, r->stream));
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    r->dtype = dtype;
    r->dims[0] = d;
    r->dims[1] = h;
    r->dims[2] = w;
    r->value_scale = value_scale;
    for (int a = 0; a < 3; ++a) {
        r->bmin[a] = min_bounds[a];
        r->bmax[a] = max_bounds[a];
    }
    r->has_volume = true;
    r->has_normals = false;
    cudaFree(r->d_nrm);
    r->d_nrm = nullptr;
    r->nrm_bytes = 0;
    r->layout_dirty = true;
    return PVR_OK;
}

int pvr_load_normals(pvr_renderer *r, const float *normals) {
    if (int rc = check_handle(r)) return rc;
    if (!normals) {
        if (r->has_normals) r->layout_dirty = true;
        r->has_normals = false;
        return PVR_OK;
    }
    if (!r->has_volume) return fail(PVR_ERR_STATE, "load a volume before its normals");
    DeviceScope ds(r->device);
    size_t bytes = (size_t)r->dims[0] * r->dims[1] * r->dims[2] * 3 * sizeof(float);
    if (bytes != r->nrm_bytes) {
        PVR_CUDA(cudaStreamSynchronize(r->stream));
        cudaFree(r->d_nrm);
        r->d_nrm = nullptr;
        r->nrm_bytes = 0;
        PVR_CUDA(cudaMalloc(&r->d_nrm, bytes));
        r->nrm_bytes = bytes;
    }
    PVR_CUDA(cudaMemcpyAsync(r->d_nrm, normals, bytes, cudaMemcpyHostToDevice, r->stream));
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    r->has_normals = true;
    r->layout_dirty = true;
    return PVR_OK;
}

int pvr_set_lut(pvr_renderer *r, const float *rgba, int size) {
    if (int rc = check_handle(r)) return rc;
    if (!rgba) return fail(PVR_ERR_VALUE, "LUT is NULL");
    if (size <= 0 || size > (1 << 24)) return fail(PVR_ERR_VALUE, "LUT size must be in 1..2^24, got %d", size);
    DeviceScope ds(r->device);
    if (size > r->lut_cap) {
        PVR_CUDA(cudaStreamSynchronize(r->stream));
        cudaFree(r->d_lut);
        r->d_lut = nullptr;
        r->lut_cap = 0;
        PVR_CUDA(cudaMalloc(&r->d_lut, (size_t)size * sizeof(float4)));
        r->lut_cap = size;
    }
    if (size + 1 > r->prefix_cap) {
        cudaFree(r->d_prefix);
        r->d_prefix = nullptr;
        r->prefix_cap = 0;
        PVR_CUDA(cudaMalloc(&r->d_prefix, (size_t)(size + 1) * sizeof(int)));
        r->prefix_cap = size + 1;
    }
    // prefix[i] = entries before i that a skipped sample must not read:
    // alpha not exactly 0, or a non-finite colour
    std::vector<int> prefix(size + 1, 0);
    for (int i = 0; i < size; ++i) {
        const float *e = rgba + 4 * i;
        bool clear = e[3] == 0.0f && std::isfinite(e[0]) && std::isfinite(e[1]) && std::isfinite(e[2]);
        prefix[i + 1] = prefix[i] + (clear ? 0 : 1);
    }
    PVR_CUDA(cudaMemcpyAsync(r->d_lut, rgba, (size_t)size * sizeof(float4), cudaMemcpyHostToDevice,
                             r->stream));
    PVR_CUDA(cudaMemcpyAsync(r->d_prefix, prefix.data(), (size_t)(size + 1) * sizeof(int),
                             cudaMemcpyHostToDevice, r->stream));
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    r->lut_size = size;
    r->flags_dirty = true;
    return PVR_OK;
}

int pvr_frame_constants(const float view[16], const float proj[16], const float light_pos[3],
                        const float light_target[3], const float min_bounds[3],
                        const float max_bounds[3], float step_size, float reference_step_size,
                        float out[27]) {
    if (!view || !proj || !light_pos || !light_target || !min_bounds || !max_bounds || !out)
        return fail(PVR_ERR_VALUE, "NULL argument");
    double ip[16], iv[16];
    if (!invert_gl(proj, ip)) return fail(PVR_ERR_VALUE, "projection matrix is singular");
    if (!invert_gl(view, iv)) return fail(PVR_ERR_VALUE, "view matrix is singular");
    for (int i = 0; i < 8; ++i) out[i] = (float)ip[i];
    for (int i = 0; i < 12; ++i) out[8 + i] = (float)iv[i];
    light_direction(light_pos, light_target, out + 20);
    for (int a = 0; a < 3; ++a) out[23 + a] = 1.0f / (max_bounds[a] - min_bounds[a]);
    out[26] = step_size / reference_step_size;
    return PVR_OK;
}

int pvr_set_camera(pvr_renderer *r, const float view[16], const float proj[16],
                   const float camera_pos[3]) {
    if (int rc = check_handle(r)) return rc;
    if (!view || !proj || !camera_pos) return fail(PVR_ERR_VALUE, "camera arrays must not be NULL");
    double ip[16], iv[16];
    if (!invert_gl(proj, ip)) return fail(PVR_ERR_VALUE, "projection matrix is singular");
    if (!invert_gl(view, iv)) return fail(PVR_ERR_VALUE, "view matrix is singular");
    for (int i = 0; i < 8; ++i) r->ip[i] = (float)ip[i];
    for (int i = 0; i < 12; ++i) r->iv[i] = (float)iv[i];
    for (int a = 0; a < 3; ++a) r->cam[a] = camera_pos[a];
    r->has_camera = true;
    return PVR_OK;
}

int pvr_set_light(pvr_renderer *r, const float position[3], const float target[3], float ambient,
                  float diffuse) {
    if (int rc = check_handle(r)) return rc;
    if (!position || !target) return fail(PVR_ERR_VALUE, "light vectors must not be NULL");
    for (int a = 0; a < 3; ++a) {
        r->light_pos[a] = position[a];
        r->light_target[a] = target[a];
    }
    r->ambient = ambient;
    r->diffuse = diffuse;
    r->flags_dirty = true;
    return PVR_OK;
}

int pvr_set_config(pvr_renderer *r, float step_size, int max_steps, float reference_step_size) {
    if (int rc = check_handle(r)) return rc;
    if (!(step_size > 0.0f) || !std::isfinite(step_size))
        return fail(PVR_ERR_VALUE, "step_size must be positive");
    if (max_steps < 1) return fail(PVR_ERR_VALUE, "max_steps must be at least 1");
    if (!(reference_step_size > 0.0f) || !std::isfinite(reference_step_size))
        return fail(PVR_ERR_VALUE, "reference_step_size must be positive");
    r->step = step_size;
    r->max_steps = max_steps;
    r->ref_step = reference_step_size;
    return PVR_OK;
}

int pvr_render(pvr_renderer *r, uint8_t *out_rgba8, float *out_rgba32f) {
    if (int rc = check_handle(r)) return rc;
    if (!out_rgba8 && !out_rgba32f) return fail(PVR_ERR_VALUE, "no output buffer given");
    DeviceScope ds(r->device);
    if (int rc = ensure_targets(r, out_rgba32f != nullptr)) return rc;
    if (int rc = march_into(r, r->d_out8, out_rgba32f ? r->d_outf : nullptr, r->stream)) return rc;
    size_t npx = (size_t)r->width * r->height;
    if (out_rgba8)
        PVR_CUDA(cudaMemcpyAsync(out_rgba8, r->d_out8, npx * 4, cudaMemcpyDeviceToHost, r->stream));
    if (out_rgba32f)
        PVR_CUDA(cudaMemcpyAsync(out_rgba32f, r->d_outf, npx * 16, cudaMemcpyDeviceToHost, r->stream));
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    return PVR_OK;
}

int pvr_render_device(pvr_renderer *r, void *d_rgba8, void *d_rgba32f, void *stream) {
    if (int rc = check_handle(r)) return rc;
    DeviceScope ds(r->device);
    if (int rc = ensure_targets(r, false)) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : r->stream;
    return march_into(r, (uint32_t *)d_rgba8, (float4 *)d_rgba32f, st);
}

int pvr_last_sample_count(pvr_renderer *r, long long *samples) {
    if (int rc = check_handle(r)) return rc;
    if (!samples) return fail(PVR_ERR_VALUE, "samples is NULL");
    DeviceScope ds(r->device);
    unsigned long long v = 0;
    PVR_CUDA(cudaDeviceSynchronize());
    PVR_CUDA(cudaMemcpy(&v, r->d_samples, sizeof(v), cudaMemcpyDeviceToHost));
    *samples = (long long)v;
    return PVR_OK;
}

int pvr_last_sample_counts(pvr_renderer *r, long long *inbox, long long *shaded) {
    if (int rc = check_handle(r)) return rc;
    if (!inbox || !shaded) return fail(PVR_ERR_VALUE, "output pointer is NULL");
    DeviceScope ds(r->device);
    unsigned long long v[2] = {0, 0};
    PVR_CUDA(cudaDeviceSynchronize());
    PVR_CUDA(cudaMemcpy(v, r->d_samples, sizeof(v), cudaMemcpyDeviceToHost));
    *inbox = (long long)v[0];
    *shaded = (long long)v[1];
    return PVR_OK;
}

int pvr_device_bytes(pvr_renderer *r, long long *bytes) {
    if (int rc = check_handle(r)) return rc;
    if (!bytes) return fail(PVR_ERR_VALUE, "bytes is NULL");
    size_t npx = (size_t)r->width * r->height;
    size_t b = r->vol_bytes + r->nrm_bytes + r->records_bytes +
               (size_t)r->geo.nbricks * (sizeof(uint32_t) + sizeof(float2)) +
               (size_t)r->lut_cap * sizeof(float4) + (size_t)r->prefix_cap * sizeof(int) + npx * 4 +
               (r->d_outf ? npx * 16 : 0) + 2 * sizeof(unsigned long long);
    *bytes = (long long)b;
    return PVR_OK;
}

}  // extern "C"
