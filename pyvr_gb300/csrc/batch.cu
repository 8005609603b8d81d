// Batched rendering: many renders in one persistent kernel launch.
//
// A launcher owns `slots` launch slots.  Each slot has its own work counter
// and a CUDA graph [zero the counter -> persistent march kernel] built once
// per launch configuration (brick size, tuning, grid, LUT staging size).
// Queuing a batch writes the job table into the kernel node's parameters
// (cudaGraphExecKernelNodeSetParams) and launches the slot's graph; a slot
// is reused only after the event recorded behind its last launch has
// completed, so up to `slots` batches can be in flight.  Batches of more
// than kMaxLaunchJobs jobs are split over consecutive launches.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "pvr_internal.h"

namespace pvr {
const void *batch_kernel_b2(const Tuning &, int);
const void *batch_kernel_b3(const Tuning &, int);
const void *batch_kernel_b4(const Tuning &, int);
const void *single_kernel_b2(const Tuning &, int);
const void *single_kernel_b3(const Tuning &, int);
const void *single_kernel_b4(const Tuning &, int);
int max_batch_blocks_b2(const Tuning &, int, int);
int max_batch_blocks_b3(const Tuning &, int, int);
int max_batch_blocks_b4(const Tuning &, int, int);

const void *batch_kernel(int log2b, const Tuning &t, int variant) {
    switch (log2b) {
    case 2: return batch_kernel_b2(t, variant);
    case 4: return batch_kernel_b4(t, variant);
    default: return batch_kernel_b3(t, variant);
    }
}

const void *single_kernel(int log2b, const Tuning &t, int variant) {
    switch (log2b) {
    case 2: return single_kernel_b2(t, variant);
    case 4: return single_kernel_b4(t, variant);
    default: return single_kernel_b3(t, variant);
    }
}

size_t batch_smem_bytes(int lut_smem_entries) {
    return (size_t)lut_smem_entries * sizeof(float4) + (size_t)(lut_smem_entries + 1) * sizeof(int);
}

int max_batch_blocks_per_sm(int log2b, const Tuning &t, int lut_smem_entries, int variant) {
    switch (log2b) {
    case 2: return max_batch_blocks_b2(t, lut_smem_entries, variant);
    case 4: return max_batch_blocks_b4(t, lut_smem_entries, variant);
    default: return max_batch_blocks_b3(t, lut_smem_entries, variant);
    }
}

int job_variant_of(const pvr_job &j, bool fast) {
    return (j.volume->normals_mode != PVR_NORMALS_NONE ? kSingleNormals : 0) |
           (j.lut->size <= kMaxSmemLut ? kSingleSmemLut : 0) | (j.volume->compact ? kSingleCompact : 0) |
           (fast ? kSingleFast : 0);
}
}  // namespace pvr

namespace {

struct LaunchKey {
    const void *fn = nullptr;
    int grid = 0, lut_smem = 0;
    bool operator==(const LaunchKey &o) const { return fn == o.fn && grid == o.grid && lut_smem == o.lut_smem; }
};

struct Slot {
    int *d_work = nullptr;
    cudaEvent_t done = nullptr;
    bool pending = false;
    cudaGraph_t graph = nullptr;  // kept: its kernel node is updated per batch
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t kernel_node = nullptr;
    LaunchKey key;
};

}  // namespace

struct pvr_batch {
    int device = 0;
    int cap = 0;
    int next = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    pvr::Tuning tuning;
    std::vector<Slot> slots;
    std::unique_ptr<pvr::BatchParams> params;  // host staging of one launch's job table
    pvr::SingleParams single;                  // ... of a one-job launch
};

using pvr::fail;

namespace {

void destroy_slot(Slot &s) {
    if (s.done) cudaEventSynchronize(s.done);
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.graph) cudaGraphDestroy(s.graph);
    if (s.done) cudaEventDestroy(s.done);
    cudaFree(s.d_work);
    s = Slot();
}

bool valid_tuning(const pvr::Tuning &t) {
    return t.tile_w > 0 && t.tile_h > 0 && t.tile_w % 8 == 0 && t.tile_h % 4 == 0 &&
           t.tile_w * t.tile_h == pvr::kBatchThreads && (t.steps_per_iter == 1 || t.steps_per_iter == 4) &&
           t.blocks_per_sm >= 0 && t.blocks_per_sm <= 16;
}

cudaKernelNodeParams kernel_params(const LaunchKey &key, void **args) {
    cudaKernelNodeParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.func = const_cast<void *>(key.fn);
    kp.gridDim = dim3(key.grid);
    kp.blockDim = dim3(pvr::kBatchThreads);
    kp.sharedMemBytes = (unsigned)pvr::batch_smem_bytes(key.lut_smem);
    kp.kernelParams = args;
    kp.extra = nullptr;
    return kp;
}

// [memset(work) -> kernel] for this slot and launch configuration
int build_graph(Slot &s, const LaunchKey &key, void **args) {
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.graph) cudaGraphDestroy(s.graph);
    s.exec = nullptr;
    s.graph = nullptr;
    s.kernel_node = nullptr;
    cudaGraph_t g = nullptr;
    PVR_CUDA(cudaGraphCreate(&g, 0));
    cudaMemsetParams mp;
    std::memset(&mp, 0, sizeof(mp));
    mp.dst = s.d_work;
    mp.value = 0;
    mp.elementSize = sizeof(int);
    mp.width = 1;
    mp.height = 1;
    cudaGraphNode_t mset = nullptr;
    cudaError_t e = cudaGraphAddMemsetNode(&mset, g, nullptr, 0, &mp);
    cudaKernelNodeParams kp = kernel_params(key, args);
    if (e == cudaSuccess) e = cudaGraphAddKernelNode(&s.kernel_node, g, &mset, 1, &kp);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&s.exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        s.exec = nullptr;
        s.kernel_node = nullptr;
        return pvr::cuda_fail(e, "batch graph");
    }
    s.graph = g;
    s.key = key;
    return PVR_OK;
}

// One launch over jobs[idx[0..n)] (jobs of one variant, at most
// kMaxLaunchJobs).
int launch_chunk(pvr_batch *b, const pvr_job *all, const int *idx, int n, bool fast, cudaStream_t st) {
    std::vector<pvr_job> jobs(n);
    for (int i = 0; i < n; ++i) jobs[i] = all[idx[i]];
    const int log2b = jobs[0].volume->log2b;
    int max_lut = 1;
    for (int i = 0; i < n; ++i) max_lut = std::max(max_lut, jobs[i].lut->size);
    Slot &s = b->slots[b->next];
    if (s.pending) {
        PVR_CUDA(cudaEventSynchronize(s.done));
        s.pending = false;
    }
    if (n == 1) {
        // one job: the single-job kernel of its variant, one block per tile,
        // launched directly (its parameters are copied at the launch, and it
        // uses no work counter); the slot's event tracks it like a batch
        pvr::SingleParams &sp = b->single;
        if (int rc = pvr::fill_job(jobs[0], b->tuning.tile_w, b->tuning.tile_h, fast, sp.job)) return rc;
        sp.tile_w = b->tuning.tile_w;
        sp.tile_h = b->tuning.tile_h;
        int lut_smem = 256;
        while (lut_smem < max_lut && lut_smem < pvr::kMaxSmemLut) lut_smem *= 2;
        sp.lut_smem_entries = lut_smem;
        const bool smem = sp.job.f.lut_size <= lut_smem;
        const int variant = (sp.job.normals ? pvr::kSingleNormals : 0) | (smem ? pvr::kSingleSmemLut : 0) |
                            (sp.job.compact ? pvr::kSingleCompact : 0) | (fast ? pvr::kSingleFast : 0);
        const long long tiles = (long long)sp.job.tiles_x * sp.job.tiles_y;
        void *args[] = {&sp};
        PVR_CUDA(cudaLaunchKernel(pvr::single_kernel(log2b, b->tuning, variant), dim3((unsigned)tiles),
                                  dim3(pvr::kBatchThreads), args, smem ? pvr::batch_smem_bytes(lut_smem) : 0,
                                  st));
        PVR_CUDA(cudaEventRecord(s.done, st));
        s.pending = true;
        b->next = (b->next + 1) % (int)b->slots.size();
        return PVR_OK;
    }
    pvr::BatchParams &p = *b->params;
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        if (int rc = pvr::fill_job(jobs[i], b->tuning.tile_w, b->tuning.tile_h, fast, p.jobs[i])) {
            const std::string why = pvr_last_error();
            return fail(rc, "job %d: %s", idx[i], why.c_str());
        }
        p.jobs[i].tile_base = (int)total;
        p.tile_base[i] = (int)total;
        total += (long long)p.jobs[i].tiles_x * p.jobs[i].tiles_y;
        if (total > (1LL << 30)) return fail(PVR_ERR_VALUE, "batch has too many tiles");
    }
    p.njobs = n;
    p.total_tiles = (int)total;
    p.tile_w = b->tuning.tile_w;
    p.tile_h = b->tuning.tile_h;
    // LUT staging sized by the largest table (a few fixed sizes so graphs are
    // reused); larger tables are read through the read-only cache
    int lut_smem = 256;
    while (lut_smem < max_lut && lut_smem < pvr::kMaxSmemLut) lut_smem *= 2;
    const int variant = pvr::job_variant(p.jobs[0]);
    if (!(variant & pvr::kSingleSmemLut)) lut_smem = 0;  // the LUTs are read from global memory
    p.lut_smem_entries = lut_smem;
    p.work = s.d_work;
    int per_sm = b->tuning.blocks_per_sm;
    const int fit = pvr::max_batch_blocks_per_sm(log2b, b->tuning, lut_smem, variant);
    if (per_sm <= 0 || per_sm > fit) per_sm = std::max(1, fit);
    LaunchKey key;
    key.fn = pvr::batch_kernel(log2b, b->tuning, variant);
    key.grid = b->sms * per_sm;
    key.lut_smem = lut_smem;
    void *args[] = {&p};
    if (!s.exec || !(s.key == key)) {
        if (int rc = build_graph(s, key, args)) return rc;
    } else {
        cudaKernelNodeParams kp = kernel_params(key, args);
        PVR_CUDA(cudaGraphExecKernelNodeSetParams(s.exec, s.kernel_node, &kp));
    }
    PVR_CUDA(cudaGraphLaunch(s.exec, st));
    PVR_CUDA(cudaEventRecord(s.done, st));
    s.pending = true;
    b->next = (b->next + 1) % (int)b->slots.size();
    return PVR_OK;
}

}  // namespace

extern "C" {

int pvr_batch_create(int capacity_jobs, int slots, pvr_batch **out) {
    if (!out) return fail(PVR_ERR_VALUE, "out is NULL");
    *out = nullptr;
    if (capacity_jobs < 1 || capacity_jobs > (1 << 16)) return fail(PVR_ERR_VALUE, "capacity must be in 1..65536");
    if (slots < 1 || slots > 16) return fail(PVR_ERR_VALUE, "slots must be in 1..16");
    pvr_batch *b = new pvr_batch();
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    b->cap = capacity_jobs;
    b->params.reset(new pvr::BatchParams());
    std::memset(b->params.get(), 0, sizeof(pvr::BatchParams));
    b->slots.resize(slots);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    for (auto &s : b->slots) {
        if (e == cudaSuccess) e = cudaMalloc(&s.d_work, sizeof(int));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        int rc = pvr::cuda_fail(e, "pvr_batch_create");
        pvr_batch_destroy(b);
        return rc;
    }
    *out = b;
    return PVR_OK;
}

int pvr_batch_destroy(pvr_batch *b) {
    if (!b) return PVR_OK;
    for (auto &s : b->slots) destroy_slot(s);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return PVR_OK;
}

int pvr_batch_set_tuning(pvr_batch *b, const pvr_tuning *tuning) {
    if (!b || !tuning) return fail(PVR_ERR_VALUE, "NULL argument");
    pvr::Tuning t;
    t.tile_w = tuning->tile_w;
    t.tile_h = tuning->tile_h;
    t.steps_per_iter = tuning->steps_per_iter;
    t.blocks_per_sm = tuning->blocks_per_sm;
    if (!valid_tuning(t))
        return fail(PVR_ERR_VALUE, "tuning: tile_w%%8==0, tile_h%%4==0, tile_w*tile_h==256, "
                                   "steps_per_iter in {1,4}, blocks_per_sm in 0..16");
    b->tuning = t;
    return PVR_OK;
}

int pvr_batch_get_tuning(const pvr_batch *b, pvr_tuning *tuning) {
    if (!b || !tuning) return fail(PVR_ERR_VALUE, "NULL argument");
    tuning->tile_w = b->tuning.tile_w;
    tuning->tile_h = b->tuning.tile_h;
    tuning->steps_per_iter = b->tuning.steps_per_iter;
    tuning->blocks_per_sm = b->tuning.blocks_per_sm;
    return PVR_OK;
}

int pvr_batch_render(pvr_batch *b, const pvr_job *jobs, int n, void *stream) {
    if (!b) return fail(PVR_ERR_VALUE, "null batch handle");
    if (n < 0 || n > b->cap) return fail(PVR_ERR_VALUE, "batch of %d jobs exceeds capacity %d", n, b->cap);
    if (n > 0 && !jobs) return fail(PVR_ERR_VALUE, "jobs is NULL");
    if (n == 0) return PVR_OK;
    const int log2b = jobs[0].volume ? jobs[0].volume->log2b : pvr::kDefaultBrickLog2;
    for (int i = 0; i < n; ++i) {
        if (!jobs[i].volume || !jobs[i].lut) return fail(PVR_ERR_VALUE, "job %d without volume or LUT", i);
        if (jobs[i].volume->log2b != log2b)
            return fail(PVR_ERR_VALUE, "all volumes of a batch must share one brick size");
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
    // volumes whose layout may still run (pvr_volume_create_async)
    for (int i = 0; i < n; ++i)
        if (i == 0 || jobs[i].volume != jobs[i - 1].volume) pvr::volume_stream_wait(jobs[i].volume, st);
    const bool fast = pvr::arithmetic_fast();  // one arithmetic for the whole call
    // one launch (or more, of at most kMaxLaunchJobs) per kernel variant
    std::vector<int> groups[16];
    for (int i = 0; i < n; ++i) groups[pvr::job_variant_of(jobs[i], fast)].push_back(i);
    for (auto &g : groups)
        for (size_t i0 = 0; i0 < g.size(); i0 += pvr::kMaxLaunchJobs)
            if (int rc = launch_chunk(b, jobs, g.data() + i0,
                                      (int)std::min<size_t>(pvr::kMaxLaunchJobs, g.size() - i0), fast, st))
                return rc;
    return PVR_OK;
}

int pvr_batch_synchronize(pvr_batch *b) {
    if (!b) return fail(PVR_ERR_VALUE, "null batch handle");
    for (auto &s : b->slots)
        if (s.pending) {
            PVR_CUDA(cudaEventSynchronize(s.done));
            s.pending = false;
        }
    return PVR_OK;
}

}  // extern "C"
