// Batched rendering: many renders in one persistent kernel launch.
//
// A launcher owns `slots` staging areas.  Each slot is a pinned host block
// and a device block holding {BatchHeader, tile bases, JobDesc[capacity]},
// a work counter, and a CUDA graph captured once per launch configuration:
// [copy host block -> device block, zero the work counter, persistent march
// kernel].  Queuing a batch fills the next slot's pinned block and launches
// its graph; a slot is reused only after the event recorded behind its last
// graph launch has completed, so up to `slots` batches can be in flight.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "pvr_internal.h"

namespace pvr {
cudaError_t launch_march_batch_b2(const Tuning &, const BatchHeader *, const int *, const JobDesc *, int *,
                                  int, int, cudaStream_t);
cudaError_t launch_march_batch_b3(const Tuning &, const BatchHeader *, const int *, const JobDesc *, int *,
                                  int, int, cudaStream_t);
cudaError_t launch_march_batch_b4(const Tuning &, const BatchHeader *, const int *, const JobDesc *, int *,
                                  int, int, cudaStream_t);
int max_batch_blocks_b2(const Tuning &, int);
int max_batch_blocks_b3(const Tuning &, int);
int max_batch_blocks_b4(const Tuning &, int);

cudaError_t launch_march_batch(int log2b, const Tuning &t, const BatchHeader *hdr, const int *tile_bases,
                               const JobDesc *jobs, int *work, int grid, int lut_smem_entries,
                               cudaStream_t st) {
    switch (log2b) {
    case 2: return launch_march_batch_b2(t, hdr, tile_bases, jobs, work, grid, lut_smem_entries, st);
    case 4: return launch_march_batch_b4(t, hdr, tile_bases, jobs, work, grid, lut_smem_entries, st);
    default: return launch_march_batch_b3(t, hdr, tile_bases, jobs, work, grid, lut_smem_entries, st);
    }
}

int max_batch_blocks_per_sm(int log2b, const Tuning &t, int lut_smem_entries) {
    switch (log2b) {
    case 2: return max_batch_blocks_b2(t, lut_smem_entries);
    case 4: return max_batch_blocks_b4(t, lut_smem_entries);
    default: return max_batch_blocks_b3(t, lut_smem_entries);
    }
}
}  // namespace pvr

namespace {

struct LaunchKey {
    int log2b = -1, tile_w = 0, tile_h = 0, steps = 0, grid = 0, lut_smem = 0;
    bool operator==(const LaunchKey &o) const {
        return log2b == o.log2b && tile_w == o.tile_w && tile_h == o.tile_h && steps == o.steps &&
               grid == o.grid && lut_smem == o.lut_smem;
    }
};

struct Slot {
    void *h_block = nullptr;  // pinned
    void *d_block = nullptr;
    int *d_work = nullptr;
    cudaEvent_t done = nullptr;
    bool pending = false;
    cudaGraphExec_t exec = nullptr;
    LaunchKey key;
};

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

}  // namespace

struct pvr_batch {
    int device = 0;
    int cap = 0;
    int next = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    pvr::Tuning tuning;
    std::vector<Slot> slots;
    size_t off_bases = 0, off_jobs = 0, block_bytes = 0;
};

using pvr::fail;

namespace {

int destroy_slot(Slot &s) {
    if (s.done) cudaEventSynchronize(s.done);
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.done) cudaEventDestroy(s.done);
    cudaFreeHost(s.h_block);
    cudaFree(s.d_block);
    cudaFree(s.d_work);
    s = Slot();
    return PVR_OK;
}

bool valid_tuning(const pvr::Tuning &t) {
    return t.tile_w > 0 && t.tile_h > 0 && t.tile_w % 8 == 0 && t.tile_h % 4 == 0 &&
           t.tile_w * t.tile_h == pvr::kBatchThreads && (t.steps_per_iter == 1 || t.steps_per_iter == 4) &&
           t.blocks_per_sm >= 0 && t.blocks_per_sm <= 16;
}

int capture(pvr_batch *b, Slot &s, const LaunchKey &key) {
    if (s.exec) {
        cudaGraphExecDestroy(s.exec);
        s.exec = nullptr;
    }
    const auto *hdr = (const pvr::BatchHeader *)s.d_block;
    const auto *bases = (const int *)((const char *)s.d_block + b->off_bases);
    const auto *jobs = (const pvr::JobDesc *)((const char *)s.d_block + b->off_jobs);
    pvr::Tuning t = b->tuning;
    PVR_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemcpyAsync(s.d_block, s.h_block, b->block_bytes, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.d_work, 0, sizeof(int), b->stream);
    if (e == cudaSuccess)
        e = pvr::launch_march_batch(key.log2b, t, hdr, bases, jobs, s.d_work, key.grid, key.lut_smem, b->stream);
    cudaGraph_t graph = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return pvr::cuda_fail(e, "batch capture");
    }
    if (e2 != cudaSuccess) return pvr::cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&s.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        s.exec = nullptr;
        return pvr::cuda_fail(e, "cudaGraphInstantiate");
    }
    s.key = key;
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
    b->off_bases = align16(sizeof(pvr::BatchHeader));
    b->off_jobs = align16(b->off_bases + sizeof(int) * capacity_jobs);
    b->block_bytes = b->off_jobs + sizeof(pvr::JobDesc) * capacity_jobs;
    b->slots.resize(slots);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    for (auto &s : b->slots) {
        if (e == cudaSuccess) e = cudaMallocHost(&s.h_block, b->block_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&s.d_block, b->block_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&s.d_work, sizeof(int));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
        if (e == cudaSuccess) std::memset(s.h_block, 0, b->block_bytes);
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
    int max_lut = 1;
    for (int i = 0; i < n; ++i) {
        if (!jobs[i].volume || !jobs[i].lut) return fail(PVR_ERR_VALUE, "job %d without volume or LUT", i);
        if (jobs[i].volume->log2b != log2b)
            return fail(PVR_ERR_VALUE, "all volumes of a batch must share one brick size");
        max_lut = std::max(max_lut, jobs[i].lut->size);
    }
    Slot &s = b->slots[b->next];
    if (s.pending) {
        PVR_CUDA(cudaEventSynchronize(s.done));
        s.pending = false;
    }
    // fill the pinned block
    auto *hdr = (pvr::BatchHeader *)s.h_block;
    int *bases = (int *)((char *)s.h_block + b->off_bases);
    auto *descs = (pvr::JobDesc *)((char *)s.h_block + b->off_jobs);
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        if (int rc = pvr::fill_job(jobs[i], b->tuning.tile_w, b->tuning.tile_h, descs[i])) {
            const std::string why = pvr_last_error();
            return fail(rc, "job %d: %s", i, why.c_str());
        }
        descs[i].tile_base = (int)total;
        bases[i] = (int)total;
        total += (long long)descs[i].tiles_x * descs[i].tiles_y;
        if (total > (1LL << 30)) return fail(PVR_ERR_VALUE, "batch has too many tiles");
    }
    hdr->njobs = n;
    hdr->total_tiles = (int)total;
    hdr->tile_w = b->tuning.tile_w;
    hdr->tile_h = b->tuning.tile_h;
    // launch configuration: LUT staging sized by the largest table (a few
    // fixed sizes so graphs are reused), persistent grid
    int lut_smem = 256;
    while (lut_smem < max_lut && lut_smem < 2048) lut_smem *= 2;
    int per_sm = b->tuning.blocks_per_sm;
    const int fit = pvr::max_batch_blocks_per_sm(log2b, b->tuning, lut_smem);
    if (per_sm <= 0 || per_sm > fit) per_sm = std::max(1, fit);
    LaunchKey key;
    key.log2b = log2b;
    key.tile_w = b->tuning.tile_w;
    key.tile_h = b->tuning.tile_h;
    key.steps = b->tuning.steps_per_iter;
    key.grid = b->sms * per_sm;
    key.lut_smem = lut_smem;
    if (!s.exec || !(s.key == key)) {
        if (int rc = capture(b, s, key)) return rc;
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
    PVR_CUDA(cudaGraphLaunch(s.exec, st));
    PVR_CUDA(cudaEventRecord(s.done, st));
    s.pending = true;
    b->next = (b->next + 1) % (int)b->slots.size();
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
