// Native serving runtime: continuous batching of render requests over
// resident volumes and LUTs, with no Python on the request path.
//
// Threads:
//  * submitters (any host thread): pvr_server_submit validates a request and
//    appends it to the queue;
//  * the scheduler: whenever a launch slot is free and requests are queued,
//    takes up to max_batch of them, and with batch_pixels > 0 only while
//    their pixels sum to at most batch_pixels (requests that arrived while
//    others were on the GPU join the next launch), and queues [march ->
//    each image to its pinned destination (or the slot's pinned arena) ->
//    event -> completion callback] on the slot's stream;
//  * the completer: takes the slots whose work has finished, in the order
//    they finish (a stream callback behind each slot's read-back hands the
//    slot over and stamps the completion time), copies each image to its
//    request's host buffer if it was staged, publishes completion records,
//    then frees the slot.  A long render does not hold back the slots that
//    finish after it was launched but before it ends.
// Up to `slots` batches are in flight, each slot on its own stream: their
// marches overlap on the device, and one batch's read-back overlaps the next
// batch's march.  With max_batch = 1 every request is its own launch, and the
// requests in flight overlap as concurrent kernels.
//
// per_frame mode is the per-frame baseline on the same machinery: one slot,
// one request per launch, and the next launch only after the previous
// request's image is in host memory.
//
// Volumes and LUTs stay owned by the caller, who keeps each alive until the
// completions of the requests that use it have been polled.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pvr_internal.h"

extern "C" int pvr_camera_spherical(const float target[3], double azimuth, double elevation, double roll,
                                    double distance, const float init_pos[3], const float init_up[3],
                                    double fov, double near_plane, double far_plane, double aspect,
                                    float view_out[16], float proj_out[16], float pos_out[3]);

namespace {

long long now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Req {
    pvr_request r;
    long long t_submit;
    long long t_launch;
};

struct Slot {
    pvr_server *srv = nullptr;  // for the completion callback
    int index = 0;
    long long t_done = 0;           // set by the completion callback
    cudaError_t stream_status = cudaSuccess;
    cudaStream_t stream = nullptr;
    pvr_batch *batch = nullptr;
    cudaEvent_t done = nullptr, k0 = nullptr, k1 = nullptr;
    void *d_arena = nullptr;
    void *h_arena = nullptr;
    size_t cap = 0, hcap = 0;
    unsigned long long *d_counters = nullptr;
    unsigned long long *h_counters = nullptr;
    std::vector<Req> reqs;
    std::vector<size_t> offs;
    std::vector<pvr_job> jobs;
    int status = PVR_OK;
    bool instrumented = false;  // this batch records kernel events and counters
};

int bytes_per_sample(int dtype) {
    return 8 * (dtype == PVR_U8 ? 1 : dtype == PVR_F16 ? 2 : 4) + 8 * 12;
}

}  // namespace

struct pvr_server {
    pvr_server_config cfg;
    int device = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_sched, cv_done, cv_poll;
    std::deque<Req> queue;
    long long queued_pixels = 0;  // width*height summed over the queue
    std::deque<int> done_slots;  // slots whose work has finished, in that order
    int n_inflight = 0;          // launched slots not yet completed
    std::vector<int> free_slots;
    std::deque<pvr_completion> completions;
    bool stop = false;
    bool paused = false;
    bool sched_exited = false;
    std::thread sched, completer;
    pvr_server_stats stats;
    std::string last_error;
    long long batch_seq = 0;  // batches launched (scheduler thread only)
};

using pvr::fail;

namespace {

// The slot's device image arena grows in stream order (no host
// synchronisation: the old arena is freed behind the work already queued).
int ensure_arena(Slot &s, size_t need) {
    if (need <= s.cap) return PVR_OK;
    size_t cap = 32u << 20;  // 24 images of 512^2 or 8 of 1024^2 before any growth
    while (cap < need) cap <<= 1;
    if (s.d_arena) PVR_CUDA(cudaFreeAsync(s.d_arena, s.stream));
    s.d_arena = nullptr;
    s.cap = 0;
    PVR_CUDA(cudaMallocAsync(&s.d_arena, cap, s.stream));
    s.cap = cap;
    return PVR_OK;
}

// The pinned staging arena, for destinations that are not page-locked only.
// The slot is idle when the scheduler fills it, so the old arena is free.
int ensure_host_arena(Slot &s, size_t need) {
    if (need <= s.hcap) return PVR_OK;
    size_t cap = 32u << 20;
    while (cap < need) cap <<= 1;
    if (s.h_arena) cudaFreeHost(s.h_arena);
    s.h_arena = nullptr;
    s.hcap = 0;
    PVR_CUDA(cudaHostAlloc(&s.h_arena, cap, cudaHostAllocPortable));
    s.hcap = cap;
    return PVR_OK;
}

void fill_from_request(const pvr_request &r, pvr_job &j) {
    std::memset(&j, 0, sizeof(j));
    j.volume = r.volume;
    j.lut = r.lut;
    j.width = r.width;
    j.height = r.height;
    std::memcpy(j.view, r.view, sizeof(j.view));
    std::memcpy(j.proj, r.proj, sizeof(j.proj));
    std::memcpy(j.camera_pos, r.camera_pos, sizeof(j.camera_pos));
    std::memcpy(j.light_pos, r.light_pos, sizeof(j.light_pos));
    std::memcpy(j.light_target, r.light_target, sizeof(j.light_target));
    j.ambient = r.ambient;
    j.diffuse = r.diffuse;
    j.step_size = r.step_size;
    j.reference_step_size = r.reference_step_size;
    j.max_steps = r.max_steps;
}

// Stream callback behind a slot's read-back: the slot's work has finished
// (or the stream has failed).  No CUDA calls are allowed here.
void CUDART_CB slot_finished(cudaStream_t, cudaError_t status, void *user) {
    Slot &s = *static_cast<Slot *>(user);
    s.t_done = now_ns();
    s.stream_status = status;
    {
        std::lock_guard<std::mutex> g(s.srv->mu);
        s.srv->done_slots.push_back(s.index);
    }
    s.srv->cv_done.notify_one();
}

// the scheduler's half of one batch: returns the status of the launch
int launch_slot(pvr_server *srv, Slot &s) {
    const int n = (int)s.reqs.size();
    // the persistent kernel drains one tile queue in job order: the most
    // expensive renders (pixels x samples per unit length) go first, so that
    // no long render starts at the end of the launch
    std::stable_sort(s.reqs.begin(), s.reqs.end(), [](const Req &a, const Req &b) {
        return (double)a.r.width * a.r.height / a.r.step_size > (double)b.r.width * b.r.height / b.r.step_size;
    });
    s.offs.resize(n);
    s.jobs.resize(n);
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        s.offs[i] = total;
        total += ((size_t)s.reqs[i].r.width * s.reqs[i].r.height * 4 + 255) & ~(size_t)255;
    }
    if (int rc = ensure_arena(s, total)) return rc;
    s.instrumented = srv->cfg.instrument > 0 && srv->batch_seq % srv->cfg.instrument == 0;
    ++srv->batch_seq;
    for (int i = 0; i < n; ++i) {
        void *ev = s.reqs[i].r.wait_event;
        bool seen = false;  // one wait per distinct event
        for (int k = 0; k < i && !seen; ++k) seen = s.reqs[k].r.wait_event == ev;
        if (ev && !seen) PVR_CUDA(cudaStreamWaitEvent(s.stream, (cudaEvent_t)ev, 0));
        // a volume whose layout may still run (pvr_volume_create_async)
        if (i == 0 || s.reqs[i].r.volume != s.reqs[i - 1].r.volume)
            pvr::volume_stream_wait(s.reqs[i].r.volume, s.stream);
    }
    for (int i = 0; i < n; ++i) {
        fill_from_request(s.reqs[i].r, s.jobs[i]);
        s.jobs[i].d_rgba8 = (char *)s.d_arena + s.offs[i];
        s.jobs[i].d_counters = s.instrumented ? s.d_counters + 2 * i : nullptr;
    }
    if (s.instrumented) {
        PVR_CUDA(cudaMemsetAsync(s.d_counters, 0, sizeof(unsigned long long) * 2 * n, s.stream));
        PVR_CUDA(cudaEventRecord(s.k0, s.stream));
    }
    if (int rc = pvr_batch_render(s.batch, s.jobs.data(), n, s.stream)) return rc;
    if (s.instrumented) {
        PVR_CUDA(cudaEventRecord(s.k1, s.stream));
        PVR_CUDA(cudaMemcpyAsync(s.h_counters, s.d_counters, sizeof(unsigned long long) * 2 * n,
                                 cudaMemcpyDeviceToHost, s.stream));
    }
    // page-locked destinations get their image by DMA; the others through
    // the slot's pinned arena and a host copy in the completer
    bool staged = false;
    for (int i = 0; i < n; ++i) {
        const pvr_request &r = s.reqs[i].r;
        if (r.out_pinned)
            PVR_CUDA(cudaMemcpyAsync(r.out_rgba8, (const char *)s.d_arena + s.offs[i], (size_t)r.width * r.height * 4,
                                     cudaMemcpyDeviceToHost, s.stream));
        else
            staged = true;
    }
    if (staged) {
        if (int rc = ensure_host_arena(s, total)) return rc;
        PVR_CUDA(cudaMemcpyAsync(s.h_arena, s.d_arena, total, cudaMemcpyDeviceToHost, s.stream));
    }
    PVR_CUDA(cudaEventRecord(s.done, s.stream));
    // last: a failed launch returns before this, and is handed over by the
    // scheduler instead
    PVR_CUDA(cudaStreamAddCallback(s.stream, slot_finished, &s, 0));
    return PVR_OK;
}

void scheduler_loop(pvr_server *srv) {
    cudaSetDevice(srv->device);
    const long long linger_ns = (long long)srv->cfg.linger_us * 1000;
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        // after stop, the queue is drained before the scheduler exits
        if (srv->stop && srv->queue.empty()) break;
        if ((srv->paused && !srv->stop) || srv->queue.empty() || srv->free_slots.empty()) {
            srv->cv_sched.wait(lk);
            continue;
        }
        // with a batch already on the GPU, a partial batch may wait up to
        // linger_us (from its oldest request's submission) for more requests
        if (!srv->cfg.per_frame && linger_ns > 0 && !srv->stop && srv->n_inflight > 0 &&
            (int)srv->queue.size() < srv->cfg.max_batch &&
            (srv->cfg.batch_pixels <= 0 || srv->queued_pixels < srv->cfg.batch_pixels)) {
            const long long due = srv->queue.front().t_submit + linger_ns;
            if (now_ns() < due) {
                srv->cv_sched.wait_until(lk, std::chrono::steady_clock::time_point(std::chrono::nanoseconds(due)));
                continue;
            }
        }
        const int si = srv->free_slots.back();
        srv->free_slots.pop_back();
        srv->n_inflight += 1;  // before the launch: its callback may run at once
        Slot &s = srv->slots[si];
        s.reqs.clear();
        const int cap = srv->cfg.per_frame ? 1 : srv->cfg.max_batch;
        long long px = 0;
        while (!srv->queue.empty() && (int)s.reqs.size() < cap) {
            const Req &q = srv->queue.front();
            const long long p = (long long)q.r.width * q.r.height;
            if (!s.reqs.empty() && srv->cfg.batch_pixels > 0 && px + p > srv->cfg.batch_pixels) break;
            px += p;
            srv->queued_pixels -= p;
            s.reqs.push_back(q);
            srv->queue.pop_front();
        }
        lk.unlock();
        const long long t_launch = now_ns();
        for (auto &q : s.reqs) q.t_launch = t_launch;
        // the slot's fields are written before its completion callback is
        // queued; a successful launch leaves them untouched afterwards
        s.stream_status = cudaSuccess;
        s.status = PVR_OK;
        const int rc = launch_slot(srv, s);
        if (rc != PVR_OK) {
            // whatever part of the batch was queued finishes before the slot
            // is handed over
            const std::string why = pvr_last_error();
            cudaStreamSynchronize(s.stream);
            s.status = rc;
            s.t_done = now_ns();
            {
                std::lock_guard<std::mutex> g(srv->mu);
                srv->last_error = why;
                srv->done_slots.push_back(si);
            }
            srv->cv_done.notify_one();
        }
        lk.lock();
    }
    srv->sched_exited = true;
    srv->cv_done.notify_all();
}

void completer_loop(pvr_server *srv) {
    cudaSetDevice(srv->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        srv->cv_done.wait(lk, [&] {
            return !srv->done_slots.empty() || (srv->sched_exited && srv->n_inflight == 0);
        });
        if (srv->done_slots.empty()) break;  // the scheduler has exited and nothing is in flight
        const int si = srv->done_slots.front();
        srv->done_slots.pop_front();
        lk.unlock();
        Slot &s = srv->slots[si];
        int status = s.status;
        if (status == PVR_OK && s.stream_status != cudaSuccess)
            status = pvr::cuda_fail(s.stream_status, "batch completion");
        const long long t_done = s.t_done;
        std::vector<pvr_completion> out(s.reqs.size());
        long long inbox = 0, shaded = 0;
        double alg = 0.0;
        float kms = 0.0f;
        for (size_t i = 0; i < s.reqs.size(); ++i) {
            const pvr_request &r = s.reqs[i].r;
            if (status == PVR_OK && !r.out_pinned)
                std::memcpy(r.out_rgba8, (const char *)s.h_arena + s.offs[i], (size_t)r.width * r.height * 4);
            out[i].tag = r.tag;
            out[i].status = status;
            out[i].t_submit_ns = s.reqs[i].t_submit;
            out[i].t_launch_ns = s.reqs[i].t_launch;
            out[i].t_done_ns = t_done;
            if (status == PVR_OK && s.instrumented) {
                inbox += (long long)s.h_counters[2 * i];
                shaded += (long long)s.h_counters[2 * i + 1];
                alg += (double)s.h_counters[2 * i + 1] * bytes_per_sample(r.volume->dtype);
            }
        }
        if (status == PVR_OK && s.instrumented) cudaEventElapsedTime(&kms, s.k0, s.k1);
        lk.lock();
        srv->stats.batches += 1;
        srv->stats.jobs += (long long)s.reqs.size();
        srv->stats.max_jobs = std::max(srv->stats.max_jobs, (int)s.reqs.size());
        srv->stats.kernel_ms += kms;
        srv->stats.inbox_samples += inbox;
        srv->stats.shaded_samples += shaded;
        srv->stats.algorithmic_bytes += alg;
        if (s.instrumented) {
            srv->stats.instrumented_batches += 1;
            srv->stats.instrumented_jobs += (long long)s.reqs.size();
        }
        for (auto &c : out) srv->completions.push_back(c);
        s.reqs.clear();
        srv->n_inflight -= 1;
        srv->free_slots.push_back(si);
        srv->cv_sched.notify_one();
        srv->cv_poll.notify_all();
    }
}

void destroy_slots(pvr_server *srv) {
    for (auto &s : srv->slots) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        if (s.batch) pvr_batch_destroy(s.batch);
        if (s.d_arena) cudaFree(s.d_arena);
        if (s.h_arena) cudaFreeHost(s.h_arena);
        if (s.d_counters) cudaFree(s.d_counters);
        if (s.h_counters) cudaFreeHost(s.h_counters);
        if (s.done) cudaEventDestroy(s.done);
        if (s.k0) cudaEventDestroy(s.k0);
        if (s.k1) cudaEventDestroy(s.k1);
        if (s.stream) cudaStreamDestroy(s.stream);
        s = Slot();
    }
}

}  // namespace

extern "C" {

int pvr_server_create(const pvr_server_config *cfg, pvr_server **out) {
    if (!cfg || !out) return fail(PVR_ERR_VALUE, "NULL argument");
    *out = nullptr;
    if (cfg->max_batch < 1 || cfg->max_batch > 4096) return fail(PVR_ERR_VALUE, "max_batch must be in 1..4096");
    if (cfg->slots < 1 || cfg->slots > 16) return fail(PVR_ERR_VALUE, "slots must be in 1..16");
    if (cfg->batch_pixels < 0) return fail(PVR_ERR_VALUE, "batch_pixels must be >= 0");
    pvr_server *srv = new pvr_server();
    srv->cfg = *cfg;
    if (srv->cfg.per_frame) {
        srv->cfg.slots = 1;
        srv->cfg.max_batch = 1;
    }
    std::memset(&srv->stats, 0, sizeof(srv->stats));
    cudaGetDevice(&srv->device);
    srv->slots.resize(srv->cfg.slots);
    int rc = PVR_OK;
    for (auto &s : srv->slots) {
        // at the highest priority, like volume layouts: renders of resident
        // volumes go ahead of other work queued on the device
        int prio_low = 0, prio_high = 0;
        cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
        cudaError_t e = cudaStreamCreateWithPriority(&s.stream, cudaStreamNonBlocking, prio_high);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreate(&s.k0);
        if (e == cudaSuccess) e = cudaEventCreate(&s.k1);
        if (e == cudaSuccess)
            e = cudaMalloc(&s.d_counters, sizeof(unsigned long long) * 2 * srv->cfg.max_batch);
        if (e == cudaSuccess)
            e = cudaHostAlloc(&s.h_counters, sizeof(unsigned long long) * 2 * srv->cfg.max_batch,
                              cudaHostAllocPortable);
        if (e != cudaSuccess) {
            rc = pvr::cuda_fail(e, "pvr_server_create");
            break;
        }
        if ((rc = pvr_batch_create(srv->cfg.max_batch, 1, &s.batch))) break;
        if (cfg->tuning.tile_w && (rc = pvr_batch_set_tuning(s.batch, &cfg->tuning))) break;
    }
    if (rc != PVR_OK) {
        destroy_slots(srv);
        delete srv;
        return rc;
    }
    for (int i = 0; i < srv->cfg.slots; ++i) {
        srv->slots[i].srv = srv;
        srv->slots[i].index = i;
    }
    for (int i = srv->cfg.slots - 1; i >= 0; --i) srv->free_slots.push_back(i);
    srv->sched = std::thread(scheduler_loop, srv);
    srv->completer = std::thread(completer_loop, srv);
    *out = srv;
    return PVR_OK;
}

int pvr_server_submit(pvr_server *srv, const pvr_request *req) {
    if (!srv || !req) return fail(PVR_ERR_VALUE, "NULL argument");
    const pvr_request &r = *req;
    if (!r.volume || !r.lut) return fail(PVR_ERR_VALUE, "request without volume or LUT");
    if (!r.volume->layout_ready) return fail(PVR_ERR_STATE, "volume layout not built");
    if (!r.out_rgba8) return fail(PVR_ERR_VALUE, "request without output buffer");
    if (r.width <= 0 || r.height <= 0 || r.width > 32768 || r.height > 32768)
        return fail(PVR_ERR_VALUE, "request size must be in 1..32768, got %dx%d", r.width, r.height);
    if (!(r.step_size > 0.0f) || !(r.reference_step_size > 0.0f) || r.max_steps < 1)
        return fail(PVR_ERR_VALUE, "invalid step_size / reference_step_size / max_steps");
    Req q;
    q.r = r;
    if (r.camera_mode == PVR_CAMERA_ORBIT) {
        if (int rc = pvr_camera_spherical(r.target, r.azimuth, r.elevation, r.roll, r.distance, r.init_pos,
                                          r.init_up, r.fov, r.near_plane, r.far_plane,
                                          (double)r.width / (double)r.height, q.r.view, q.r.proj,
                                          q.r.camera_pos))
            return rc;
    } else if (r.camera_mode != PVR_CAMERA_MATRICES) {
        return fail(PVR_ERR_VALUE, "unknown camera_mode %d", r.camera_mode);
    }
    q.t_submit = now_ns();
    {
        std::lock_guard<std::mutex> g(srv->mu);
        if (srv->stop) return fail(PVR_ERR_STATE, "server is shutting down");
        srv->queue.push_back(q);
        srv->queued_pixels += (long long)r.width * r.height;
        srv->stats.submitted += 1;
    }
    srv->cv_sched.notify_one();
    return PVR_OK;
}

int pvr_server_poll(pvr_server *srv, pvr_completion *out, int max, int timeout_ms, int *n_out) {
    if (!srv || !out || !n_out || max < 1) return fail(PVR_ERR_VALUE, "invalid poll arguments");
    *n_out = 0;
    std::unique_lock<std::mutex> lk(srv->mu);
    if (srv->completions.empty() && timeout_ms > 0)
        srv->cv_poll.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !srv->completions.empty(); });
    int n = 0;
    while (n < max && !srv->completions.empty()) {
        out[n++] = srv->completions.front();
        srv->completions.pop_front();
    }
    *n_out = n;
    return PVR_OK;
}

int pvr_server_pause(pvr_server *srv, int paused) {
    if (!srv) return fail(PVR_ERR_VALUE, "NULL argument");
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->paused = paused != 0;
    }
    srv->cv_sched.notify_all();
    return PVR_OK;
}

int pvr_server_get_stats(pvr_server *srv, pvr_server_stats *out) {
    if (!srv || !out) return fail(PVR_ERR_VALUE, "NULL argument");
    std::lock_guard<std::mutex> g(srv->mu);
    *out = srv->stats;
    out->queued = (long long)srv->queue.size();
    return PVR_OK;
}

int pvr_server_reset_stats(pvr_server *srv) {
    if (!srv) return fail(PVR_ERR_VALUE, "NULL argument");
    std::lock_guard<std::mutex> g(srv->mu);
    std::memset(&srv->stats, 0, sizeof(srv->stats));
    return PVR_OK;
}

const char *pvr_server_last_error(pvr_server *srv) {
    if (!srv) return "null server";
    std::lock_guard<std::mutex> g(srv->mu);
    thread_local std::string copy;
    copy = srv->last_error;
    return copy.c_str();
}

int pvr_server_destroy(pvr_server *srv) {
    if (!srv) return PVR_OK;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->stop = true;
    }
    // the scheduler drains the queue before it exits; the completer drains
    // the launched slots
    srv->cv_sched.notify_all();
    if (srv->sched.joinable()) srv->sched.join();
    srv->cv_done.notify_all();
    if (srv->completer.joinable()) srv->completer.join();
    destroy_slots(srv);
    delete srv;
    return PVR_OK;
}

}  // extern "C"
