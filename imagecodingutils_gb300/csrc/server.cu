// server.cu -- continuous-batching request loop for sequence jobs
// (motion estimation + transform), no vpp counterpart.
//
// A request is one sequence: nframes host luma planes of one size.  For every
// frame pair (t-1, t) the job estimates the Full-search vectors, forms the
// motion-compensated luma residual, runs the 4x4 transform + quantisation +
// dequantisation + inverse round trip on it (inter rounding at the request's
// QP) and returns the vectors and a digest of levels and reconstruction.
// Each frame is uploaded once and stays on the device as the next pair's
// reference.
//
// Scheduling: `slots` worker threads, each with its own stream and its own
// estimators (one per frame geometry, kept across requests).  A worker takes
// the oldest queued request whose device buffers fit under the memory budget
// (buffers are stream-ordered allocations, released when the request
// completes), so requests arriving while others run are admitted as soon as a
// slot and memory free up, and their kernels overlap the running ones on the
// device.  Latency is measured from submit to the completion of the
// request's last copy.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "me_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

__global__ void k_digest(const short* __restrict__ lev, const short* __restrict__ rec, long long n,
                         unsigned long long* out)
{
    long long acc = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        acc += (long long)lev[i] + 3 * (long long)rec[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, (unsigned long long)acc);
}

// Fold one estimate's status bits into the request's (the estimator's control
// block is reset by the next estimate).
__global__ void k_fold_status(const int* __restrict__ st, int* acc) { *acc |= *st; }

struct Job {
    unsigned long long ticket;
    vppgpu_seq_request req;
    size_t bytes;  // device buffers while it runs
    Clock::time_point submitted;
};

struct Done {
    unsigned long long ticket;
    int status;
    double latency_ms;
};

size_t job_bytes(const vppgpu_seq_request& r)
{
    const size_t plane = (size_t)r.width * r.height * sizeof(short);
    const size_t nmb = (size_t)(r.width / 16) * (r.height / 16);
    // two resident frames, residual, levels, reconstruction, vectors, digests,
    // status word (256-byte aligned)
    return 5 * (plane + 256) + nmb * 4 + 256 + 8 * (size_t)r.nframes + 4 + 4096;
}

}  // namespace

struct vppgpu_server {
    vppgpu_ctx* parent;
    int nslots;
    unsigned long long budget;
    unsigned long long reserved = 0, reserved_peak = 0;
    int running = 0, running_peak = 0;
    bool stop = false;
    unsigned long long next_ticket = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job> queue;
    std::vector<Done> done;
    std::vector<std::thread> workers;
    struct Slot {
        vppgpu_ctx* ctx = nullptr;
        int* h_status = nullptr;  // pinned
        std::unique_ptr<std::mutex> pool_mu{new std::mutex};  // the worker vs vppgpu_server_prepare
        struct Entry {
            int W, H, range;
            vppgpu_me* me;
        };
        std::vector<Entry> pool;
    };
    std::vector<Slot> slots;
};

namespace {

int slot_estimator(vppgpu_server::Slot& sl, int W, int H, int range, vppgpu_me** out)
{
    std::lock_guard<std::mutex> lk(*sl.pool_mu);
    for (auto& e : sl.pool)
        if (e.W == W && e.H == H && e.range == range) {
            *out = e.me;
            return VPPGPU_OK;
        }
    vppgpu_me* me = nullptr;
    int rc = vppgpu_me_create(sl.ctx, VPPGPU_ME_FULL, W, H, range, &me);
    if (rc) return rc;
    sl.pool.push_back({W, H, range, me});
    *out = me;
    return VPPGPU_OK;
}

// One sequence on one slot; returns the first non-zero status.
int run_job(vppgpu_server::Slot& sl, const vppgpu_seq_request& r)
{
    vppgpu_ctx* ctx = sl.ctx;
    cudaStream_t st = ctx->stream;
    const int W = r.width, H = r.height, nmb = (W / 16) * (H / 16);
    const size_t plane = (size_t)W * H * sizeof(short);
    vppgpu_me* me = nullptr;
    int rc = slot_estimator(sl, W, H, r.motion_range, &me);
    if (rc) return rc;
    // sub-buffers at 256-byte boundaries (16-byte stores, 64-bit atomics)
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t pl = up(plane), off_mv = 5 * pl, off_dig = off_mv + up((size_t)nmb * 4);
    const size_t off_st = off_dig + 8 * (size_t)r.nframes, bytes = off_st + 4;
    unsigned char* buf = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&buf, bytes, st));
    short* frame[2] = {(short*)buf, (short*)(buf + pl)};
    short* res = (short*)(buf + 2 * pl);
    short* lev = (short*)(buf + 3 * pl);
    short* rec = (short*)(buf + 4 * pl);
    short* mv = (short*)(buf + off_mv);
    unsigned long long* dig = (unsigned long long*)(buf + off_dig);
    int* stat = (int*)(buf + off_st);
    VPP_CUDA(cudaMemsetAsync(dig, 0, 8 * (size_t)r.nframes + 4, st));
    VPP_CUDA(cudaMemcpyAsync(frame[0], r.frames, plane, cudaMemcpyHostToDevice, st));
    for (int t = 1; t < r.nframes && !rc; t++) {
        short* cur = frame[t & 1];
        short* ref = frame[(t - 1) & 1];
        VPP_CUDA(cudaMemcpyAsync(cur, r.frames + (size_t)t * W * H, plane, cudaMemcpyHostToDevice, st));
        if ((rc = vppgpu_me_estimate_device(me, cur, ref, nullptr, nullptr, mv, nullptr, nullptr))) break;
        k_fold_status<<<1, 1, 0, st>>>(vppgpu::me_status_word(me), stat);
        if ((rc = vppgpu_me_residual_device(me, mv, res))) break;
        const int rows = H / 16;  // rows below the last full macroblock row carry no residual
        if ((rc = vppgpu_tq_roundtrip_plane_device(ctx, res, lev, rec, W, 16 * rows, W, r.qp, 0,
                                                   VPPGPU_INV_ROWS_FIRST, nullptr)))
            break;
        const long long n = (long long)W * 16 * rows;
        k_digest<<<ctx->sm_count * 2, 256, 0, st>>>(lev, rec, n, dig + (t - 1));
        if (cudaGetLastError() != cudaSuccess) {
            rc = VPPGPU_ERR_CUDA;
            break;
        }
        ctx->launches += 2;
        if (r.mv_out)
            VPP_CUDA(cudaMemcpyAsync(r.mv_out + (size_t)(t - 1) * nmb * 2, mv, (size_t)nmb * 4,
                                     cudaMemcpyDeviceToHost, st));
    }
    if (!rc && r.digest_out && r.nframes > 1)
        VPP_CUDA(cudaMemcpyAsync(r.digest_out, dig, 8 * (size_t)(r.nframes - 1), cudaMemcpyDeviceToHost, st));
    *sl.h_status = 0;
    if (!rc) VPP_CUDA(cudaMemcpyAsync(sl.h_status, stat, 4, cudaMemcpyDeviceToHost, st));
    cudaFreeAsync(buf, st);
    VPP_CUDA(cudaStreamSynchronize(st));
    if (!rc) rc = vppgpu::status_from_bits(*sl.h_status);
    return rc;
}

void worker(vppgpu_server* s, int slot)
{
    cudaSetDevice(s->parent->device);
    for (;;) {
        Job job;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            // the oldest request whose buffers fit under the budget
            s->cv_work.wait(lk, [&] {
                return (s->stop && s->queue.empty()) ||
                       (!s->queue.empty() && s->reserved + s->queue.front().bytes <= s->budget);
            });
            if (s->stop && s->queue.empty()) return;
            if (s->queue.empty() || s->reserved + s->queue.front().bytes > s->budget) continue;
            job = s->queue.front();
            s->queue.pop_front();
            s->reserved += job.bytes;
            if (s->reserved > s->reserved_peak) s->reserved_peak = s->reserved;
            s->running++;
            if (s->running > s->running_peak) s->running_peak = s->running;
        }
        const int st = run_job(s->slots[slot], job.req);
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - job.submitted).count();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->reserved -= job.bytes;
            s->running--;
            s->done.push_back({job.ticket, st, ms});
        }
        s->cv_work.notify_all();
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

int vppgpu_server_create(vppgpu_ctx* ctx, int slots, unsigned long long hbm_budget, vppgpu_server** out)
{
    if (!ctx || !out || slots < 1 || slots > 64) return VPPGPU_ERR_INVALID_ARG;
    *out = nullptr;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    if (!hbm_budget) {  // default: half of the memory free now
        size_t fr = 0, tot = 0;
        VPP_CUDA(cudaMemGetInfo(&fr, &tot));
        hbm_budget = fr / 2;
    }
    {
        // keep freed request buffers in the stream-ordered pool up to the
        // budget instead of returning them at every synchronisation
        cudaMemPool_t pool;
        VPP_CUDA(cudaDeviceGetDefaultMemPool(&pool, ctx->device));
        uint64_t keep = hbm_budget;
        VPP_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    vppgpu_server* s = new (std::nothrow) vppgpu_server();
    if (!s) return VPPGPU_ERR_OUT_OF_MEMORY;
    s->parent = ctx;
    s->nslots = slots;
    s->budget = hbm_budget;
    s->slots.resize(slots);
    for (int i = 0; i < slots; i++) {
        if (!rc && (rc = vppgpu_ctx_create(ctx->device, &s->slots[i].ctx))) s->slots[i].ctx = nullptr;
        if (!rc && cudaMallocHost((void**)&s->slots[i].h_status, sizeof(int)) != cudaSuccess) {
            s->slots[i].h_status = nullptr;
            rc = VPPGPU_ERR_OUT_OF_MEMORY;
        }
    }
    if (rc) {
        for (auto& sl : s->slots) {
            if (sl.h_status) cudaFreeHost(sl.h_status);
            if (sl.ctx) vppgpu_ctx_destroy(sl.ctx);
        }
        delete s;
        return rc;
    }
    for (int i = 0; i < slots; i++) s->workers.emplace_back(worker, s, i);
    *out = s;
    return VPPGPU_OK;
}

int vppgpu_server_prepare(vppgpu_server* s, int width, int height, int motion_range)
{
    if (!s || width < 16 || height < 16 || (width % 16) || motion_range < 4) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(s->parent);
    if (rc) return rc;
    for (auto& sl : s->slots) {
        vppgpu_me* me = nullptr;
        if ((rc = slot_estimator(sl, width, height, motion_range, &me))) return rc;
    }
    return VPPGPU_OK;
}

int vppgpu_server_submit(vppgpu_server* s, const vppgpu_seq_request* r, unsigned long long* ticket)
{
    if (!s || !r || !r->frames || r->nframes < 1 || r->width < 16 || r->height < 16 || (r->width % 16) ||
        r->qp < 0 || r->qp > 51)
        return VPPGPU_ERR_INVALID_ARG;
    Job j;
    j.req = *r;
    j.bytes = job_bytes(*r);
    j.submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (j.bytes > s->budget) return VPPGPU_ERR_OUT_OF_MEMORY;
        j.ticket = s->next_ticket++;
        s->queue.push_back(j);
    }
    if (ticket) *ticket = j.ticket;
    s->cv_work.notify_one();
    return VPPGPU_OK;
}

int vppgpu_server_poll(vppgpu_server* s, int max, unsigned long long* tickets, int* status, double* latency_ms,
                       int* n)
{
    if (!s || !n || max < 0) return VPPGPU_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    const int k = (int)s->done.size() < max ? (int)s->done.size() : max;
    for (int i = 0; i < k; i++) {
        if (tickets) tickets[i] = s->done[i].ticket;
        if (status) status[i] = s->done[i].status;
        if (latency_ms) latency_ms[i] = s->done[i].latency_ms;
    }
    s->done.erase(s->done.begin(), s->done.begin() + k);
    *n = k;
    return VPPGPU_OK;
}

int vppgpu_server_wait_idle(vppgpu_server* s)
{
    if (!s) return VPPGPU_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->queue.empty() && s->running == 0; });
    return VPPGPU_OK;
}

int vppgpu_server_stats(vppgpu_server* s, unsigned long long* reserved_peak, int* running_peak)
{
    if (!s) return VPPGPU_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (reserved_peak) *reserved_peak = s->reserved_peak;
    if (running_peak) *running_peak = s->running_peak;
    return VPPGPU_OK;
}

int vppgpu_server_destroy(vppgpu_server* s)
{
    if (!s) return VPPGPU_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    cudaSetDevice(s->parent->device);
    for (auto& sl : s->slots) {
        for (auto& e : sl.pool) vppgpu_me_destroy(e.me);
        cudaFreeHost(sl.h_status);
        vppgpu_ctx_destroy(sl.ctx);
    }
    delete s;
    return VPPGPU_OK;
}

}  // extern "C"
