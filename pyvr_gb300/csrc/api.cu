// C ABI of the renderer handle: the job of pyvr's ModernGLManager
// (pyvr/moderngl_renderer/manager.py) and of the uniform plumbing of
// ModernGLVolumeRenderer (renderer.py:303-316), on CUDA device buffers.
// A render is a batch of one job on the persistent march kernel.
#include <cmath>
#include <cstring>

#include "pvr_internal.h"

using pvr::fail;

struct pvr_renderer {
    int device = 0;
    int width = 0, height = 0;
    cudaStream_t stream = nullptr;
    pvr_volume *vol = nullptr;  // owned: load_volume / load_normals
    pvr_lut *lut = nullptr;     // owned: set_transfer_functions
    pvr_batch *batch = nullptr;
    // camera uniforms as sent by renderer.py:160-172
    bool has_camera = false;
    float view[16] = {}, proj[16] = {}, cam[3] = {};
    // light + config uniforms (Light.default(), RenderConfig.balanced())
    float light_pos[3] = {1.0f, 1.0f, 1.0f}, light_target[3] = {0.0f, 0.0f, 0.0f};
    float ambient = 0.2f, diffuse = 0.8f;
    float step = 0.01f, ref_step = 0.01f;
    int max_steps = 500;
    // render targets
    uint32_t *d_out8 = nullptr;
    float4 *d_outf = nullptr;
    uint8_t *h_out8 = nullptr;  // page-locked image of pvr_render_pinned
    unsigned long long *d_counters = nullptr;  // [in-box samples, shaded samples]
};

namespace {

size_t dtype_size(int dtype) { return dtype == PVR_U8 ? 1 : dtype == PVR_F16 ? 2 : 4; }

bool finite3(const float v[3]) {
    return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

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

int check_handle(pvr_renderer *r) {
    if (!r) return fail(PVR_ERR_VALUE, "null renderer handle");
    return PVR_OK;
}

// wait for every render queued by this handle
int quiesce(pvr_renderer *r) {
    if (r->batch)
        if (int rc = pvr_batch_synchronize(r->batch)) return rc;
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    return PVR_OK;
}

void drop_volume(pvr_renderer *r) {
    if (!r->vol) return;
    pvr_volume_destroy(r->vol);
    r->vol = nullptr;
}

int ensure_targets(pvr_renderer *r, bool want_float) {
    const size_t npx = (size_t)r->width * r->height;
    if (!r->d_out8) PVR_CUDA(cudaMalloc(&r->d_out8, npx * 4));
    if (want_float && !r->d_outf) PVR_CUDA(cudaMalloc(&r->d_outf, npx * 16));
    if (!r->d_counters) PVR_CUDA(cudaMalloc(&r->d_counters, 2 * sizeof(unsigned long long)));
    return PVR_OK;
}

int march_into(pvr_renderer *r, uint32_t *d8, float4 *df, cudaStream_t st) {
    PVR_CUDA(cudaMemsetAsync(r->d_counters, 0, 2 * sizeof(unsigned long long), st));
    if (!r->vol) {  // unbound samplers read zero: transparent image
        const size_t npx = (size_t)r->width * r->height;
        if (d8) PVR_CUDA(cudaMemsetAsync(d8, 0, npx * 4, st));
        if (df) PVR_CUDA(cudaMemsetAsync(df, 0, npx * 16, st));
        return PVR_OK;
    }
    if (!r->has_camera) return fail(PVR_ERR_STATE, "Camera not set: call set_camera() before render()");
    if (!r->lut)
        return fail(PVR_ERR_STATE, "Transfer functions not set: call set_transfer_functions() before render()");
    if (int rc = pvr::ensure_volume_layout(r->vol, r->stream)) return rc;
    pvr_job j;
    std::memset(&j, 0, sizeof(j));
    j.volume = r->vol;
    j.lut = r->lut;
    j.width = r->width;
    j.height = r->height;
    std::memcpy(j.view, r->view, sizeof(j.view));
    std::memcpy(j.proj, r->proj, sizeof(j.proj));
    std::memcpy(j.camera_pos, r->cam, sizeof(j.camera_pos));
    std::memcpy(j.light_pos, r->light_pos, sizeof(j.light_pos));
    std::memcpy(j.light_target, r->light_target, sizeof(j.light_target));
    j.ambient = r->ambient;
    j.diffuse = r->diffuse;
    j.step_size = r->step;
    j.reference_step_size = r->ref_step;
    j.max_steps = r->max_steps;
    j.d_rgba8 = d8;
    j.d_rgba32f = df;
    j.d_counters = r->d_counters;
    return pvr_batch_render(r->batch, &j, 1, st);
}

}  // namespace

extern "C" {

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
        return pvr::cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    int rc = pvr_batch_create(1, 1, &r->batch);
    if (rc == PVR_OK) rc = ensure_targets(r, false);
    if (rc != PVR_OK) {
        pvr_destroy(r);
        return rc;
    }
    *out = r;
    return PVR_OK;
}

int pvr_destroy(pvr_renderer *r) {
    if (!r) return PVR_OK;
    DeviceScope ds(r->device);
    quiesce(r);
    drop_volume(r);
    pvr_lut_destroy(r->lut);
    pvr_batch_destroy(r->batch);
    cudaFree(r->d_out8);
    cudaFree(r->d_outf);
    cudaFree(r->d_counters);
    cudaFreeHost(r->h_out8);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
    return PVR_OK;
}

int pvr_load_volume(pvr_renderer *r, const void *data, int dtype, int d, int h, int w, float value_scale,
                    const float min_bounds[3], const float max_bounds[3]) {
    if (int rc = check_handle(r)) return rc;
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
    DeviceScope ds(r->device);
    if (int rc = quiesce(r)) return rc;
    drop_volume(r);
    pvr_volume *v = new pvr_volume();
    v->device = r->device;
    v->dtype = dtype;
    v->dims[0] = d;
    v->dims[1] = h;
    v->dims[2] = w;
    v->value_scale = value_scale;
    for (int a = 0; a < 3; ++a) {
        v->bmin[a] = min_bounds[a];
        v->bmax[a] = max_bounds[a];
    }
    v->vol_bytes = (size_t)d * h * w * dtype_size(dtype);
    cudaError_t e = pvr::vol_alloc(&v->d_vol, v->vol_bytes, r->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v->d_vol, data, v->vol_bytes, cudaMemcpyHostToDevice, r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    if (e != cudaSuccess) {
        pvr::vol_free(v->d_vol, r->stream);
        cudaStreamSynchronize(r->stream);
        delete v;
        return pvr::cuda_fail(e, "upload volume");
    }
    r->vol = v;  // records are built at the first render
    return PVR_OK;
}

int pvr_load_normals(pvr_renderer *r, const float *normals) {
    if (int rc = check_handle(r)) return rc;
    if (!normals) {
        if (r->vol && r->vol->normals_mode != PVR_NORMALS_NONE) {
            if (int rc = quiesce(r)) return rc;
            r->vol->normals_mode = PVR_NORMALS_NONE;
            r->vol->layout_ready = false;
        }
        return PVR_OK;
    }
    if (!r->vol) return fail(PVR_ERR_STATE, "load a volume before its normals");
    DeviceScope ds(r->device);
    if (int rc = quiesce(r)) return rc;
    pvr_volume *v = r->vol;
    const size_t bytes = (size_t)v->dims[0] * v->dims[1] * v->dims[2] * 3 * sizeof(float);
    pvr::vol_free(v->d_nrm, r->stream);
    v->d_nrm = nullptr;
    PVR_CUDA(pvr::vol_alloc((void **)&v->d_nrm, bytes, r->stream));
    PVR_CUDA(cudaMemcpyAsync(v->d_nrm, normals, bytes, cudaMemcpyHostToDevice, r->stream));
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    v->normals_mode = PVR_NORMALS_GIVEN;
    v->layout_ready = false;
    return PVR_OK;
}

int pvr_compute_normals(pvr_renderer *r) {
    if (int rc = check_handle(r)) return rc;
    if (!r->vol) return fail(PVR_ERR_STATE, "load a volume before computing its normals");
    pvr_volume *v = r->vol;
    if (v->dims[0] < 2 || v->dims[1] < 2 || v->dims[2] < 2)
        return fail(PVR_ERR_VALUE, "Shape of array too small to calculate a numerical gradient, "
                                   "at least (edge_order + 1) elements are required.");
    DeviceScope ds(r->device);
    if (int rc = quiesce(r)) return rc;
    pvr::vol_free(v->d_nrm, r->stream);
    v->d_nrm = nullptr;
    v->normals_mode = PVR_NORMALS_DEVICE;
    v->layout_ready = false;
    return PVR_OK;
}

int pvr_set_lut(pvr_renderer *r, const float *rgba, int size) {
    if (int rc = check_handle(r)) return rc;
    DeviceScope ds(r->device);
    if (int rc = quiesce(r)) return rc;  // a queued render may still read the table
    if (!r->lut) return pvr_lut_create(rgba, size, &r->lut);
    return pvr_lut_update(r->lut, rgba, size);
}

int pvr_set_camera(pvr_renderer *r, const float view[16], const float proj[16], const float camera_pos[3]) {
    if (int rc = check_handle(r)) return rc;
    if (!view || !proj || !camera_pos) return fail(PVR_ERR_VALUE, "camera arrays must not be NULL");
    double tmp[16];
    if (!pvr::invert_gl(proj, tmp)) return fail(PVR_ERR_VALUE, "projection matrix is singular");
    if (!pvr::invert_gl(view, tmp)) return fail(PVR_ERR_VALUE, "view matrix is singular");
    std::memcpy(r->view, view, sizeof(r->view));
    std::memcpy(r->proj, proj, sizeof(r->proj));
    std::memcpy(r->cam, camera_pos, sizeof(r->cam));
    r->has_camera = true;
    return PVR_OK;
}

int pvr_set_light(pvr_renderer *r, const float position[3], const float target[3], float ambient,
                  float diffuse) {
    if (int rc = check_handle(r)) return rc;
    if (!position || !target) return fail(PVR_ERR_VALUE, "light vectors must not be NULL");
    std::memcpy(r->light_pos, position, sizeof(r->light_pos));
    std::memcpy(r->light_target, target, sizeof(r->light_target));
    r->ambient = ambient;
    r->diffuse = diffuse;
    return PVR_OK;
}

int pvr_set_config(pvr_renderer *r, float step_size, int max_steps, float reference_step_size) {
    if (int rc = check_handle(r)) return rc;
    if (!(step_size > 0.0f) || !std::isfinite(step_size)) return fail(PVR_ERR_VALUE, "step_size must be positive");
    if (max_steps < 1) return fail(PVR_ERR_VALUE, "max_steps must be at least 1");
    if (!(reference_step_size > 0.0f) || !std::isfinite(reference_step_size))
        return fail(PVR_ERR_VALUE, "reference_step_size must be positive");
    r->step = step_size;
    r->max_steps = max_steps;
    r->ref_step = reference_step_size;
    return PVR_OK;
}

int pvr_set_tuning(pvr_renderer *r, const pvr_tuning *tuning) {
    if (int rc = check_handle(r)) return rc;
    return pvr_batch_set_tuning(r->batch, tuning);
}

int pvr_render(pvr_renderer *r, uint8_t *out_rgba8, float *out_rgba32f) {
    if (int rc = check_handle(r)) return rc;
    if (!out_rgba8 && !out_rgba32f) return fail(PVR_ERR_VALUE, "no output buffer given");
    DeviceScope ds(r->device);
    if (int rc = ensure_targets(r, out_rgba32f != nullptr)) return rc;
    if (int rc = march_into(r, r->d_out8, out_rgba32f ? r->d_outf : nullptr, r->stream)) return rc;
    const size_t npx = (size_t)r->width * r->height;
    if (out_rgba8) PVR_CUDA(cudaMemcpyAsync(out_rgba8, r->d_out8, npx * 4, cudaMemcpyDeviceToHost, r->stream));
    if (out_rgba32f)
        PVR_CUDA(cudaMemcpyAsync(out_rgba32f, r->d_outf, npx * 16, cudaMemcpyDeviceToHost, r->stream));
    PVR_CUDA(cudaStreamSynchronize(r->stream));
    return PVR_OK;
}

int pvr_render_pinned(pvr_renderer *r, const uint8_t **rgba8) {
    if (!rgba8) return fail(PVR_ERR_VALUE, "rgba8 is NULL");
    *rgba8 = nullptr;
    if (int rc = check_handle(r)) return rc;
    DeviceScope ds(r->device);
    const size_t npx = (size_t)r->width * r->height;
    if (!r->h_out8) PVR_CUDA(cudaMallocHost((void **)&r->h_out8, npx * 4));
    if (int rc = pvr_render(r, r->h_out8, nullptr)) return rc;
    *rgba8 = r->h_out8;
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
    long long shaded = 0;
    return pvr_last_sample_counts(r, samples, &shaded);
}

int pvr_last_sample_counts(pvr_renderer *r, long long *inbox, long long *shaded) {
    if (int rc = check_handle(r)) return rc;
    if (!inbox || !shaded) return fail(PVR_ERR_VALUE, "output pointer is NULL");
    DeviceScope ds(r->device);
    unsigned long long v[2] = {0, 0};
    PVR_CUDA(cudaDeviceSynchronize());
    PVR_CUDA(cudaMemcpy(v, r->d_counters, sizeof(v), cudaMemcpyDeviceToHost));
    *inbox = (long long)v[0];
    *shaded = (long long)v[1];
    return PVR_OK;
}

int pvr_device_bytes(pvr_renderer *r, long long *bytes) {
    if (int rc = check_handle(r)) return rc;
    if (!bytes) return fail(PVR_ERR_VALUE, "bytes is NULL");
    const size_t npx = (size_t)r->width * r->height;
    long long b = (long long)(npx * 4 + (r->d_outf ? npx * 16 : 0) + 2 * sizeof(unsigned long long));
    if (r->vol) {
        long long vb = 0;
        pvr_volume_device_bytes(r->vol, &vb);
        b += vb;
        if (r->vol->d_nrm) b += (long long)((size_t)r->vol->dims[0] * r->vol->dims[1] * r->vol->dims[2] * 12);
    }
    if (r->lut) b += (long long)r->lut->cap * (sizeof(float4) + sizeof(int));
    *bytes = b;
    return PVR_OK;
}

}  // extern "C"
