// pvr_batch_render_static: the persistent batch march without any memory
// allocation in the call or in a handle it needs.
//
// pvr_batch_render takes a pvr_batch launcher, whose creation allocates a
// device tile counter per slot (cudaMalloc) and whose destruction frees them
// (cudaFree synchronises the whole device).  Some callers cannot do either:
// an application that hands the entire device memory to its own pool, a frame
// loop with a fixed memory budget that must not fail on an allocation half
// way through, or a host that must not add device-wide synchronisation.  This
// entry point needs only the pvr_volume / pvr_lut handles and the output
// buffers the caller already owns; the one piece of scratch memory the kernel
// needs -- a tile counter per launch, which must read 0 when the launch
// starts -- lives in a fixed static device array, cleared by the call itself
// (cudaMemsetAsync on the caller's stream) before the launches that use it.
//
// Limits and rules:
//  * at most kStaticCounters launches per call, one per kernel variant
//    (normals, record form, arithmetic) and per kMaxLaunchJobs jobs of it
//    (64 x 96 = 6144 jobs of one variant); larger calls fail with
//    PVR_ERR_VALUE before anything is queued;
//  * the counters are shared by every call on a device: two calls whose work
//    may overlap on the GPU (different streams, or different host threads
//    without ordering) race on them and can skip or repeat tiles.  Issue the
//    calls on one stream, or order them with events;
//  * the address of the static array is looked up once per device context
//    (cudaGetSymbolAddress, which also loads this module on that device):
//    on the first call on a device, and again on the first call after the
//    device's context was replaced (cudaDeviceReset); make those calls
//    outside stream capture.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "pvr_internal.h"

namespace {

constexpr int kStaticCounters = 64;  // 256 bytes of scratch per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) static int g_tile_counters[kStaticCounters];

// The array's address in one device context: a context replaced by
// cudaDeviceReset holds the module at a new address, so the cached address
// is keyed by the context's process-unique id (cuCtxGetId).
struct CounterAddr {
    unsigned long long ctx_id;
    int *ptr;
};
std::mutex g_counter_mutex;
CounterAddr g_counter_addr[kMaxDevices];

// cuCtxGetCurrent / cuCtxGetId from the driver the runtime already loaded
// (no link-time dependency on libcuda).
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

// Id of the calling thread's current context; 0 if none is current yet (the
// runtime creates the primary context lazily) or if the driver entry points
// are unavailable (then the address is cached per device alone).
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

int counters_for_device(int device, int **out) {
    if (device < 0 || device >= kMaxDevices) return pvr::fail(PVR_ERR_VALUE, "device ordinal %d out of range", device);
    std::lock_guard<std::mutex> lock(g_counter_mutex);
    CounterAddr &c = g_counter_addr[device];
    const unsigned long long ctx = current_context_id();
    if (!c.ptr || ctx == 0 || c.ctx_id != ctx) {
        // also makes the device's primary context current if it was not yet
        void *addr = nullptr;
        PVR_CUDA(cudaGetSymbolAddress(&addr, g_tile_counters));
        c.ptr = static_cast<int *>(addr);
        c.ctx_id = current_context_id();
    }
    *out = c.ptr;
    return PVR_OK;
}

bool tuning_ok(const pvr::Tuning &t) {
    return t.tile_w > 0 && t.tile_h > 0 && t.tile_w % 8 == 0 && t.tile_h % 4 == 0 &&
           t.tile_w * t.tile_h == pvr::kBatchThreads && (t.steps_per_iter == 1 || t.steps_per_iter == 4) &&
           t.blocks_per_sm >= 0 && t.blocks_per_sm <= 16;
}

}  // namespace

using pvr::fail;

extern "C" int pvr_batch_render_static(const pvr_job *jobs, int n, const pvr_tuning *tuning, void *stream) {
    constexpr int kMaxJobs = kStaticCounters * pvr::kMaxLaunchJobs;
    if (n < 0 || n > kMaxJobs)
        return fail(PVR_ERR_VALUE,
                    "pvr_batch_render_static: %d jobs; at most %d per call (%d launches of %d jobs, "
                    "one static tile counter each)",
                    n, kMaxJobs, kStaticCounters, pvr::kMaxLaunchJobs);
    if (n > 0 && !jobs) return fail(PVR_ERR_VALUE, "jobs is NULL");
    if (n == 0) return PVR_OK;
    pvr::Tuning t;
    if (tuning) {
        t.tile_w = tuning->tile_w;
        t.tile_h = tuning->tile_h;
        t.steps_per_iter = tuning->steps_per_iter;
        t.blocks_per_sm = tuning->blocks_per_sm;
        if (!tuning_ok(t))
            return fail(PVR_ERR_VALUE, "tuning: tile_w%%8==0, tile_h%%4==0, tile_w*tile_h==256, "
                                       "steps_per_iter in {1,4}, blocks_per_sm in 0..16");
    }
    if (!jobs[0].volume) return fail(PVR_ERR_VALUE, "job 0 without volume or LUT");
    const int log2b = jobs[0].volume->log2b;
    for (int i = 0; i < n; ++i) {
        if (!jobs[i].volume || !jobs[i].lut) return fail(PVR_ERR_VALUE, "job %d without volume or LUT", i);
        if (jobs[i].volume->log2b != log2b)
            return fail(PVR_ERR_VALUE, "all volumes of a batch must share one brick size");
    }
    int device = 0, sms = 0;
    PVR_CUDA(cudaGetDevice(&device));
    PVR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    int *counters = nullptr;
    if (int rc = counters_for_device(device, &counters)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const bool fast = pvr::arithmetic_fast();
    // jobs grouped by kernel variant (counting sort, on the stack): one launch
    // per variant and per kMaxLaunchJobs jobs, one static counter per launch
    constexpr int kVariants = 16;
    int order[kMaxJobs];
    int start[kVariants + 1] = {0};
    for (int i = 0; i < n; ++i) ++start[pvr::job_variant_of(jobs[i], fast) + 1];
    for (int v = 0; v < kVariants; ++v) start[v + 1] += start[v];
    {
        int next[kVariants];
        for (int v = 0; v < kVariants; ++v) next[v] = start[v];
        for (int i = 0; i < n; ++i) order[next[pvr::job_variant_of(jobs[i], fast)]++] = i;
    }
    int launches = 0;
    for (int v = 0; v < kVariants; ++v)
        launches += (start[v + 1] - start[v] + pvr::kMaxLaunchJobs - 1) / pvr::kMaxLaunchJobs;
    if (launches > kStaticCounters)
        return fail(PVR_ERR_VALUE,
                    "pvr_batch_render_static: the jobs need %d launches (one per kernel variant and per %d "
                    "jobs), at most %d per call",
                    launches, pvr::kMaxLaunchJobs, kStaticCounters);
    // job tables are built on the host stack: the launch copies its parameters
    pvr::BatchParams p;
    // validate every job before anything is queued
    for (int i = 0; i < n; ++i) {
        if (int rc = pvr::fill_job(jobs[i], t.tile_w, t.tile_h, fast, p.jobs[0])) {
            const std::string why = pvr_last_error();
            return fail(rc, "job %d: %s", i, why.c_str());
        }
    }
    // volumes whose layout may still run (pvr_volume_create_async): the
    // stream waits for them; under stream capture, whose graph cannot wait on
    // work queued outside it, every layout must have completed
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    PVR_CUDA(cudaStreamIsCapturing(st, &capture));
    for (int i = 0; i < n; ++i) {
        const pvr_volume *v = jobs[i].volume;
        if (i > 0 && v == jobs[i - 1].volume) continue;
        if (capture != cudaStreamCaptureStatusNone) {
            if (v->ready && !v->ready_done.load())
                return fail(PVR_ERR_STATE, "job %d: the volume's layout may still be running (wait for "
                                           "pvr_volume_ready before capturing)", i);
        } else {
            pvr::volume_stream_wait(v, st);
        }
    }
    for (int v = 0, c = 0; v < kVariants; ++v) {
        for (int i0 = start[v]; i0 < start[v + 1]; i0 += pvr::kMaxLaunchJobs) {
            const int m = std::min(pvr::kMaxLaunchJobs, start[v + 1] - i0);
            long long total = 0;
            int max_lut = 1;
            for (int i = 0; i < m; ++i) {
                const pvr_job &j = jobs[order[i0 + i]];
                pvr::fill_job(j, t.tile_w, t.tile_h, fast, p.jobs[i]);
                p.jobs[i].tile_base = (int)total;
                p.tile_base[i] = (int)total;
                total += (long long)p.jobs[i].tiles_x * p.jobs[i].tiles_y;
                max_lut = std::max(max_lut, j.lut->size);
            }
            if (total > (1LL << 30)) return fail(PVR_ERR_VALUE, "launch %d has too many tiles", c);
            ++c;
        }
    }
    PVR_CUDA(cudaMemsetAsync(counters, 0, (size_t)launches * sizeof(int), st));
    for (int v = 0, c = 0; v < kVariants; ++v) {
        if (start[v + 1] == start[v]) continue;
        const void *fn = pvr::batch_kernel(log2b, t, v);
        for (int i0 = start[v]; i0 < start[v + 1]; i0 += pvr::kMaxLaunchJobs, ++c) {
            const int m = std::min(pvr::kMaxLaunchJobs, start[v + 1] - i0);
            long long total = 0;
            int max_lut = 1;
            for (int i = 0; i < m; ++i) {
                const pvr_job &j = jobs[order[i0 + i]];
                pvr::fill_job(j, t.tile_w, t.tile_h, fast, p.jobs[i]);
                p.jobs[i].tile_base = (int)total;
                p.tile_base[i] = (int)total;
                total += (long long)p.jobs[i].tiles_x * p.jobs[i].tiles_y;
                max_lut = std::max(max_lut, j.lut->size);
            }
            p.njobs = m;
            p.total_tiles = (int)total;
            p.tile_w = t.tile_w;
            p.tile_h = t.tile_h;
            int lut_smem = 256;
            while (lut_smem < max_lut && lut_smem < pvr::kMaxSmemLut) lut_smem *= 2;
            if (!(v & pvr::kSingleSmemLut)) lut_smem = 0;  // the LUTs are read from global memory
            p.lut_smem_entries = lut_smem;
            p.work = counters + c;
            int per_sm = t.blocks_per_sm;
            const int fit = pvr::max_batch_blocks_per_sm(log2b, t, lut_smem, v);
            if (per_sm <= 0 || per_sm > fit) per_sm = std::max(1, fit);
            void *args[] = {&p};
            PVR_CUDA(cudaLaunchKernel(fn, dim3(sms * per_sm), dim3(pvr::kBatchThreads), args,
                                      pvr::batch_smem_bytes(lut_smem), st));
        }
    }
    return PVR_OK;
}
