// tw_server.cu -- the serving loop: many meshing jobs resident in HBM, their
// query batches joined across jobs as they arrive (include/tw_gb300.h,
// "serving loop").
//
// Jobs are data holders: each is a tw_ctx whose surfaces (LBVHs), parameters
// and resident vertex arrays are built by the single-job entry points.  Work
// runs on lanes: each lane is a private tw_ctx (its own stream, scratch and
// device counters) that borrows a job's device data for the launches of one
// batch.  A dispatcher thread owns the lanes: it reaps finished lanes,
// forms the next batch from the waiting requests (points with points, faces
// with faces, any jobs, one segment per request; AMIPS requests of any jobs
// one after another; a smoothing request alone) and launches it on a free
// lane, so batches on different lanes overlap on the device.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tw_internal.h"

using namespace tw;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxLanes = 16;
constexpr int kMaxBatchRequests = 512;
constexpr int64_t kMaxBatchQueries = int64_t(1) << 23;   // points or faces per launch
constexpr int64_t kMaxRequestItems = int64_t(1) << 27;
constexpr unsigned long long kErrBadIds = 16ULL;          // lane error bit: star ids out of range

struct Job {
    tw_ctx* c = nullptr;     // owns the job's surfaces, parameters and mesh
    int pending = 0;         // requests submitted and not yet completed
    bool smoothing = false;  // a TW_REQ_SMOOTH of this job is on a lane
    bool cancelling = false; // tw_server_job_cancel in progress: no new submissions
};

struct Req {
    uint64_t ticket = 0;
    int32_t job = -1;
    tw_ctx* jc = nullptr;    // the job's context, captured when the batch is formed
    tw_request r{};
    Clock::time_point t_submit, t_done;
    int status = TW_OK;
    bool done = false;
    std::string error;
};

struct Lane {
    tw_ctx* c = nullptr;
    cudaEvent_t done_ev = nullptr;
    std::vector<Req*> batch;
    bool busy = false;
    size_t bytes = 0;                         // lane scratch held (updated under the lock)
    void* seg_host = nullptr;                 // pinned segment records (kMaxBatchRequests)
    unsigned long long* err_host = nullptr;   // pinned copy of the lane's error word
};

void borrow(tw_ctx* lane, const tw_ctx* job) {
    lane->vx = job->vx;
    lane->vy = job->vy;
    lane->vz = job->vz;
    lane->rounded = job->rounded;
    lane->nv = job->nv;
    lane->surf[0] = job->surf[0];
    lane->surf[1] = job->surf[1];
    lane->eps2 = job->eps2;
    lane->sampling_dist = job->sampling_dist;
}

void unborrow(tw_ctx* lane) {
    lane->vx = lane->vy = lane->vz = nullptr;
    lane->rounded = nullptr;
    lane->nv = 0;
    lane->surf[0] = Surface{};
    lane->surf[1] = Surface{};
}

__global__ void k_check_ids_flag(const int32_t* __restrict__ ids, int64_t n, int32_t lim,
                                 unsigned long long* __restrict__ counters) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t v = ids[i];
    if (v < 0 || v >= lim) atomicOr(counters + kCntError, kErrBadIds);
}

__global__ void k_apply_moves(const int32_t* __restrict__ centers, const uint8_t* __restrict__ st,
                              const double* __restrict__ out, int64_t n, double* __restrict__ vx,
                              double* __restrict__ vy, double* __restrict__ vz) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || st[i] != TW_SMOOTH_MOVED) return;
    int32_t v = centers[i];
    vx[v] = out[3 * i];
    vy[v] = out[3 * i + 1];
    vz[v] = out[3 * i + 2];
}

__global__ void k_mesh_aos(const double* __restrict__ vx, const double* __restrict__ vy,
                           const double* __restrict__ vz, int32_t nv, double* __restrict__ xyz) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    xyz[3 * i] = vx[i];
    xyz[3 * i + 1] = vy[i];
    xyz[3 * i + 2] = vz[i];
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct tw_server {
    int device = 0;
    size_t budget = 0;
    std::vector<std::unique_ptr<Job>> jobs;   // stable addresses; closed jobs have c == nullptr
    std::vector<Lane> lanes;
    std::mutex mu;                            // queue, requests, jobs bookkeeping
    std::condition_variable cv;               // dispatcher wake-up and request completion
    std::mutex admin;                         // job open / close / mesh (serialised)
    std::deque<Req*> queue;
    std::unordered_map<uint64_t, Req*> reqs;
    uint64_t next_ticket = 1;
    std::thread th;
    bool stop = false;
    int precision = TW_PRECISION_FP32_CERTIFIED;
    int newton_max_step = 15, newton_max_it = 20, newton_shape = 5;
    tw_server_stats stats{};
    std::string last_error;
};

namespace {

int srv_fail(tw_server* s, int code, const std::string& msg) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->last_error = msg;
    return code;
}

// the same with s->mu already held by the caller
int srv_fail_locked(tw_server* s, int code, const std::string& msg) {
    s->last_error = msg;
    return code;
}

size_t lanes_bytes(tw_server* s) {
    size_t b = 0;
    for (auto& L : s->lanes) b += L.bytes;
    return b;
}

// Settings of one batch, copied under the lock.
struct BatchParams {
    int precision, max_step, max_it, shape;
};

size_t jobs_bytes(tw_server* s) {
    size_t b = 0;
    for (auto& j : s->jobs)
        if (j->c) b += j->c->used;
    return b;
}

Job* job_at(tw_server* s, int32_t id) {
    if (id < 0 || id >= (int32_t)s->jobs.size()) return nullptr;
    Job* j = s->jobs[id].get();
    return j->c ? j : nullptr;
}

int64_t request_queries(const tw_request& r) { return r.n; }

// ---- batch launches (dispatcher thread, lane stream) ---------------------------------
// Each returns TW_OK or an error for the whole batch; the copies back and the
// completion event are recorded by the caller.
int launch_segments(const BatchParams& P, Lane& L, std::vector<Req*>& B, int kind) {
    tw_ctx* c = L.c;
    const size_t in_sz = kind == TW_REQ_POINTS ? 24 : 72;
    int64_t n = 0;
    for (Req* q : B) n += q->r.n;
    const size_t segb = env_seg_bytes();
    const size_t bytes = align256(in_sz * (size_t)n) + align256((size_t)n) +
                         align256(segb * B.size()) + 256;
    void* p;
    int st = ensure(c, 0, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    char* din = q; q += align256(in_sz * (size_t)n);
    uint8_t* dout = (uint8_t*)q; q += align256((size_t)n);
    void* dseg = q;
    int64_t off = 0;
    for (size_t i = 0; i < B.size(); ++i) {
        const tw_request& r = B[i]->r;
        const tw_ctx* jc = B[i]->jc;
        fill_env_seg((char*)L.seg_host + i * segb, jc->surf[TW_SURFACE_INPUT], off, jc->eps2,
                     jc->sampling_dist);
        if (r.n > 0)
            cudaMemcpyAsync(din + in_sz * off, r.in0, in_sz * (size_t)r.n, cudaMemcpyHostToDevice,
                            c->stream);
        off += r.n;
    }
    cudaMemcpyAsync(dseg, L.seg_host, segb * B.size(), cudaMemcpyHostToDevice, c->stream);
    if (kind == TW_REQ_POINTS)
        launch_env_points_segs((const double*)din, n, dseg, (int)B.size(), dout, P.precision,
                               c->counters, c->stream);
    else
        launch_env_faces_segs((const double*)din, n, dseg, (int)B.size(), dout, P.precision,
                              c->counters, c->stream);
    off = 0;
    for (Req* rq : B) {
        if (rq->r.n > 0)
            cudaMemcpyAsync(rq->r.out0, dout + off, (size_t)rq->r.n, cudaMemcpyDeviceToHost,
                            c->stream);
        off += rq->r.n;
    }
    return TW_OK;
}

int launch_amips(const BatchParams& P, Lane& L, std::vector<Req*>& B) {
    tw_ctx* c = L.c;
    size_t bytes = 256;
    for (Req* q : B) bytes += align256(96 * (size_t)q->r.n) + align256(105 * (size_t)q->r.n);
    void* p;
    int st = ensure(c, 0, bytes, &p);
    if (st != TW_OK) return st;
    // the requests of a batch run one after another on the lane's stream, so
    // they share the lane's recheck list (sized for the largest)
    char* rs = nullptr;
    if (P.precision == TW_PRECISION_FP32_CERTIFIED) {
        int64_t max_n = 0;
        for (Req* rq : B) max_n = std::max<int64_t>(max_n, rq->r.n);
        if ((st = amips_recheck_scratch(c, max_n, 1, &rs)) != TW_OK) return st;
    }
    char* q = (char*)p;
    for (Req* rq : B) {
        const tw_request& r = rq->r;
        const size_t n = (size_t)r.n;
        double* dT = (double*)q; q += align256(96 * n);
        double* dE = (double*)q;
        double* dJ = dE + n;
        double* dH = dJ + 3 * n;
        uint8_t* dF = (uint8_t*)(dH + 9 * n);
        q += align256(105 * n);
        if (n == 0) continue;
        cudaMemcpyAsync(dT, r.in0, 96 * n, cudaMemcpyHostToDevice, c->stream);
        const int mode = (r.flags & TW_REQ_RAW) ? TW_ENERGY_RAW : TW_ENERGY_QUALITY;
        double* E = r.out0 ? dE : nullptr;
        double* J = r.out1 ? dJ : nullptr;
        double* H = r.out2 ? dH : nullptr;
        uint8_t* F = r.out3 ? dF : nullptr;
        if (P.precision == TW_PRECISION_FP32_CERTIFIED)
            launch_amips_soa_cert(dT, (int64_t)n, mode, E, J, H, F, c->counters, rs, c->stream,
                                  c->energy_form);
        else
            launch_amips_soa(dT, (int64_t)n, mode, E, J, H, F, c->counters + kCntExactOrient,
                             c->stream, c->energy_form);
        if (E) cudaMemcpyAsync(r.out0, dE, 8 * n, cudaMemcpyDeviceToHost, c->stream);
        if (J) cudaMemcpyAsync(r.out1, dJ, 24 * n, cudaMemcpyDeviceToHost, c->stream);
        if (H) cudaMemcpyAsync(r.out2, dH, 72 * n, cudaMemcpyDeviceToHost, c->stream);
        if (F) cudaMemcpyAsync(r.out3, dF, n, cudaMemcpyDeviceToHost, c->stream);
    }
    return TW_OK;
}

int launch_smooth(const BatchParams& P, Lane& L, Req* rq) {
    tw_ctx* c = L.c;
    const tw_request& r = rq->r;
    const int32_t ns = (int32_t)r.n;
    const int32_t* off = (const int32_t*)r.in0;
    const int64_t nt = off[ns];
    const bool any_surface = r.in4 != nullptr;
    borrow(c, rq->jc);
    c->precision = P.precision;
    c->newton_max_step = P.max_step;
    c->newton_max_it = P.max_it;
    c->newton_shape = P.shape;
    SmoothScratch S;
    int st = smooth_scratch(c, ns, nt, S);
    if (st != TW_OK) {
        unborrow(c);
        return st;
    }
    const size_t nsz = (size_t)ns;
    const size_t bytes = align256(4 * (nsz + 1)) + align256(16 * (size_t)nt) +
                         align256((size_t)nt) + align256(4 * nsz) + align256(nsz) +
                         align256(24 * nsz) + align256(nsz) + 256;
    void* p;
    st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) {
        unborrow(c);
        return st;
    }
    char* q = (char*)p;
    int32_t* doff = (int32_t*)q; q += align256(4 * (nsz + 1));
    int32_t* dt = (int32_t*)q; q += align256(16 * (size_t)nt);
    uint8_t* dff = (uint8_t*)q; q += align256((size_t)nt);
    int32_t* dc = (int32_t*)q; q += align256(4 * nsz);
    uint8_t* dk = (uint8_t*)q; q += align256(nsz);
    double* dout = (double*)q; q += align256(24 * nsz);
    uint8_t* dst = (uint8_t*)q;
    cudaMemcpyAsync(doff, off, 4 * (nsz + 1), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dt, r.in1, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    if (any_surface) cudaMemcpyAsync(dff, r.in2, (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dc, r.in3, 4 * nsz, cudaMemcpyHostToDevice, c->stream);
    if (any_surface) cudaMemcpyAsync(dk, r.in4, nsz, cudaMemcpyHostToDevice, c->stream);
    if (nt > 0)
        k_check_ids_flag<<<(unsigned)((4 * nt + 255) / 256), 256, 0, c->stream>>>(dt, 4 * nt, c->nv,
                                                                                c->counters);
    k_check_ids_flag<<<(unsigned)((nsz + 255) / 256), 256, 0, c->stream>>>(dc, ns, c->nv,
                                                                           c->counters);
    smooth_launch(c, doff, dt, any_surface ? dff : nullptr, dc, any_surface ? dk : nullptr, ns,
                  any_surface, dout, dst, S);
    if (r.flags & TW_REQ_APPLY)
        k_apply_moves<<<(unsigned)((nsz + 255) / 256), 256, 0, c->stream>>>(dc, dst, dout, ns,
                                                                           c->vx, c->vy, c->vz);
    cudaMemcpyAsync(r.out0, dout, 24 * nsz, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(r.out1, dst, nsz, cudaMemcpyDeviceToHost, c->stream);
    unborrow(c);
    return TW_OK;
}

// Takes the next batch out of the queue (caller holds mu).  Points / faces:
// requests of the kind at the front, in arrival order, up to the batch caps.
// AMIPS likewise.  Smoothing: the first smoothing request whose job has no
// smoothing pass on a lane (passes of one job stay in order).
std::vector<Req*> form_batch(tw_server* s) {
    std::vector<Req*> B;
    if (s->queue.empty()) return B;
    int kind = -1;
    for (Req* q : s->queue) {
        if (q->r.kind != TW_REQ_SMOOTH || !s->jobs[q->job]->smoothing) {
            kind = q->r.kind;
            break;
        }
    }
    if (kind < 0) return B;
    int64_t nq = 0;
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        Req* q = *it;
        bool take = false;
        if (q->r.kind == kind) {
            if (kind == TW_REQ_SMOOTH) {
                take = B.empty() && !s->jobs[q->job]->smoothing;
            } else {
                take = (int)B.size() < kMaxBatchRequests &&
                       (B.empty() || nq + q->r.n <= kMaxBatchQueries);
            }
        }
        if (take) {
            q->jc = s->jobs[q->job]->c;
            B.push_back(q);
            nq += q->r.n;
            it = s->queue.erase(it);
            if (kind == TW_REQ_SMOOTH) {
                s->jobs[q->job]->smoothing = true;
                break;
            }
        } else {
            ++it;
        }
    }
    return B;
}

void complete(tw_server* s, Lane& L, int status, const std::string& err) {
    const auto now = Clock::now();
    for (Req* q : L.batch) {
        q->status = status;
        q->error = err;
        q->t_done = now;
        q->done = true;
        Job* j = s->jobs[q->job].get();
        j->pending -= 1;
        if (q->r.kind == TW_REQ_SMOOTH) j->smoothing = false;
        s->stats.requests_done += 1;
        s->stats.queries_done += (uint64_t)request_queries(q->r);
    }
    s->stats.batches += 1;
    s->stats.max_requests_per_batch =
        std::max<uint64_t>(s->stats.max_requests_per_batch, L.batch.size());
    L.batch.clear();
    L.busy = false;
}

std::string decode_err(unsigned long long err) {
    std::string m;
    if (err & 1ULL) m += "surface traversal exceeded its bounds; ";
    if (err & 2ULL) m += "a face exceeds the per-row sample bound; ";
    if (err & 4ULL) m += "a boundary star without a boundary surface; ";
    if (err & 8ULL) m += "smoothing face list exceeded its capacity; ";
    if (err & kErrBadIds) m += "star vertex id out of range; ";
    return m;
}

void dispatcher(tw_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        bool any_busy = false;
        for (auto& L : s->lanes) {
            if (!L.busy) continue;
            cudaError_t e = cudaEventQuery(L.done_ev);
            if (e == cudaErrorNotReady) {
                any_busy = true;
                continue;
            }
            if (e != cudaSuccess) {
                complete(s, L, TW_ERR_CUDA, cudaGetErrorString(e));
            } else if (*L.err_host) {
                std::string m = decode_err(*L.err_host);
                complete(s, L, TW_ERR_ARG, m);
            } else {
                complete(s, L, TW_OK, "");
            }
            s->cv.notify_all();
        }
        if (s->stop && s->queue.empty() && !any_busy) break;
        Lane* freeL = nullptr;
        for (auto& L : s->lanes)
            if (!L.busy) {
                freeL = &L;
                break;
            }
        if (freeL && !s->queue.empty()) {
            std::vector<Req*> B = form_batch(s);
            if (!B.empty()) {
                freeL->busy = true;
                freeL->batch = B;
                const int kind = B[0]->r.kind;
                const BatchParams P{s->precision, s->newton_max_step, s->newton_max_it,
                                    s->newton_shape};
                lk.unlock();
                Lane& L = *freeL;
                tw_ctx* c = L.c;
                *L.err_host = 0;
                cudaMemsetAsync(c->counters + kCntError, 0, sizeof(unsigned long long), c->stream);
                int st;
                if (kind == TW_REQ_POINTS || kind == TW_REQ_FACES)
                    st = launch_segments(P, L, B, kind);
                else if (kind == TW_REQ_AMIPS)
                    st = launch_amips(P, L, B);
                else
                    st = launch_smooth(P, L, B[0]);
                cudaMemcpyAsync(L.err_host, c->counters + kCntError, sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, c->stream);
                cudaError_t e = cudaGetLastError();
                if (st == TW_OK && e == cudaSuccess) cudaEventRecord(L.done_ev, c->stream);
                const size_t lane_bytes = c->used;
                lk.lock();
                L.bytes = lane_bytes;
                if (st != TW_OK || e != cudaSuccess) {
                    cudaStreamSynchronize(c->stream);
                    complete(s, L, st != TW_OK ? st : TW_ERR_CUDA,
                             st != TW_OK ? c->last_error : cudaGetErrorString(e));
                    s->cv.notify_all();
                }
                continue;
            }
        }
        if (any_busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        } else {
            s->cv.wait_for(lk, std::chrono::milliseconds(50));
        }
    }
}

// Waits (mu held through lk) until the job has no pending requests.
bool drain_job(tw_server* s, std::unique_lock<std::mutex>& lk, Job* j, double timeout_s) {
    return s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                          [&] { return j->pending == 0; });
}

}  // namespace

extern "C" {

int tw_server_create(int device, size_t hbm_budget, int lanes, tw_server** out) {
    if (!out || lanes < 1 || lanes > kMaxLanes) return TW_ERR_ARG;
    *out = nullptr;
    tw_server* s = new tw_server();
    s->device = device;
    s->budget = hbm_budget;
    cudaSetDevice(device);
    for (int i = 0; i < lanes; ++i) {
        Lane L;
        int st = tw_ctx_create(device, 0, &L.c);
        if (st != TW_OK) {
            for (auto& M : s->lanes) tw_ctx_destroy(M.c);
            delete s;
            return st;
        }
        cudaEventCreateWithFlags(&L.done_ev, cudaEventDisableTiming);
        cudaHostAlloc(&L.seg_host, env_seg_bytes() * kMaxBatchRequests, cudaHostAllocDefault);
        cudaHostAlloc((void**)&L.err_host, sizeof(unsigned long long), cudaHostAllocDefault);
        if (!L.seg_host || !L.err_host) {
            cudaGetLastError();
            tw_ctx_destroy(L.c);
            for (auto& M : s->lanes) tw_ctx_destroy(M.c);
            delete s;
            return TW_ERR_OOM;
        }
        s->lanes.push_back(L);
    }
    s->th = std::thread(dispatcher, s);
    *out = s;
    return TW_OK;
}

int tw_server_destroy(tw_server* s) {
    if (!s) return TW_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->th.joinable()) s->th.join();
    cudaSetDevice(s->device);
    for (auto& L : s->lanes) {
        unborrow(L.c);
        tw_ctx_destroy(L.c);
        cudaEventDestroy(L.done_ev);
        cudaFreeHost(L.seg_host);
        cudaFreeHost(L.err_host);
    }
    for (auto& j : s->jobs)
        if (j->c) tw_ctx_destroy(j->c);
    for (auto& kv : s->reqs) delete kv.second;
    delete s;
    return TW_OK;
}

const char* tw_server_last_error(tw_server* s) { return s ? s->last_error.c_str() : ""; }

int tw_server_set_params(tw_server* s, int precision, int max_step, int max_it, int shape) {
    if (!s) return TW_ERR_ARG;
    if (precision != TW_PRECISION_FP64 && precision != TW_PRECISION_FP32_CERTIFIED)
        return srv_fail(s, TW_ERR_ARG, "unknown precision mode");
    if (max_step < 0 || max_it < 0 || shape < 0 || shape >= newton_num_shapes())
        return srv_fail(s, TW_ERR_ARG, "bad Newton parameters");
    std::lock_guard<std::mutex> lk(s->mu);
    s->precision = precision;
    s->newton_max_step = max_step;
    s->newton_max_it = max_it;
    s->newton_shape = shape;
    return TW_OK;
}

int tw_server_job_open(tw_server* s, const double* V, int32_t nv, const int32_t* F, int32_t nf,
                       double eps_2, double sampling_dist, int32_t* job) {
    if (!s || !job || nv <= 0 || nf <= 0 || !V || !F) return TW_ERR_ARG;
    std::lock_guard<std::mutex> ak(s->admin);
    // footprint: nodes (128 + 64 B), facet records (128 + 72 + 4 B) per facet,
    // build temporaries, counters
    // plus the certified-envelope grid: up to 256 cells (4 B) per facet and
    // up to ~300 list entries (4 B) per facet
    const size_t est = (420 + 1024 + 1200) * (size_t)nf + 48 * (size_t)nv + (size_t(4) << 20);
    size_t used;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        used = jobs_bytes(s) + lanes_bytes(s);
    }
    if (s->budget && used + est > s->budget)
        return srv_fail(s, TW_BUSY, "job does not fit in the HBM budget now");
    tw_ctx* c = nullptr;
    int st = tw_ctx_create(s->device, 0, &c);
    if (st != TW_OK) return srv_fail(s, st, "tw_ctx_create failed");
    // no bin index: a job's point queries read the grid's hashed cells, so the
    // footprint stays within the estimate above
    c->bin_cell = 0.0;
    st = tw_set_params(c, eps_2, sampling_dist, 15, 20);
    if (st == TW_OK) st = tw_surface_upload(c, V, nv, F, nf, TW_SURFACE_INPUT);
    if (st != TW_OK) {
        std::string m = c->last_error;
        tw_ctx_destroy(c);
        return srv_fail(s, st, "job_open: " + m);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    // the estimate admitted it; the bytes the job actually holds decide
    if (s->budget && jobs_bytes(s) + lanes_bytes(s) + c->used > s->budget) {
        tw_ctx_destroy(c);
        return srv_fail_locked(s, TW_BUSY, "job does not fit in the HBM budget now");
    }
    int32_t id = -1;
    for (size_t i = 0; i < s->jobs.size(); ++i)
        if (!s->jobs[i]->c) {
            id = (int32_t)i;
            break;
        }
    if (id < 0) {
        s->jobs.push_back(std::make_unique<Job>());
        id = (int32_t)s->jobs.size() - 1;
    }
    Job* j = s->jobs[id].get();
    j->c = c;
    j->pending = 0;
    j->smoothing = false;
    *job = id;
    return TW_OK;
}

int tw_server_job_boundary(tw_server* s, int32_t job, const double* V, int32_t nv,
                           const int32_t* F, int32_t nf) {
    if (!s) return TW_ERR_ARG;
    std::lock_guard<std::mutex> ak(s->admin);
    Job* j;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        j = job_at(s, job);
        if (!j) return srv_fail_locked(s, TW_ERR_ARG, "no such job");
        if (!drain_job(s, lk, j, 60.0)) return srv_fail_locked(s, TW_ERR_TIMEOUT, "job busy");
    }
    int st = tw_surface_upload(j->c, V, nv, F, nf, TW_SURFACE_BOUNDARY);
    return st == TW_OK ? TW_OK : srv_fail(s, st, j->c->last_error);
}

int tw_server_job_mesh(tw_server* s, int32_t job, const double* xyz, int32_t nv,
                       double timeout_s) {
    if (!s) return TW_ERR_ARG;
    std::lock_guard<std::mutex> ak(s->admin);
    Job* j;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        j = job_at(s, job);
        if (!j) return srv_fail_locked(s, TW_ERR_ARG, "no such job");
        if (!drain_job(s, lk, j, timeout_s))
            return srv_fail_locked(s, TW_ERR_TIMEOUT, "job has requests in flight");
    }
    int st = tw_mesh_upload(j->c, xyz, nv, nullptr);
    return st == TW_OK ? TW_OK : srv_fail(s, st, j->c->last_error);
}

int tw_server_job_read_mesh(tw_server* s, int32_t job, double* xyz, double timeout_s) {
    if (!s || !xyz) return TW_ERR_ARG;
    std::lock_guard<std::mutex> ak(s->admin);
    Job* j;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        j = job_at(s, job);
        if (!j) return srv_fail_locked(s, TW_ERR_ARG, "no such job");
        if (!drain_job(s, lk, j, timeout_s))
            return srv_fail_locked(s, TW_ERR_TIMEOUT, "job has requests in flight");
    }
    tw_ctx* c = j->c;
    if (!c->vx) return srv_fail(s, TW_ERR_NO_MESH, "job has no resident mesh");
    cudaSetDevice(s->device);
    void* tmp;
    int st = ensure(c, 6, 24 * (size_t)c->nv, &tmp);
    if (st != TW_OK) return srv_fail(s, st, c->last_error);
    k_mesh_aos<<<(unsigned)((c->nv + 255) / 256), 256, 0, c->stream>>>(c->vx, c->vy, c->vz, c->nv,
                                                                       (double*)tmp);
    cudaMemcpyAsync(xyz, tmp, 24 * (size_t)c->nv, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? TW_OK : srv_fail(s, TW_ERR_CUDA, cudaGetErrorString(e));
}

int tw_server_job_close(tw_server* s, int32_t job, double timeout_s) {
    if (!s) return TW_ERR_ARG;
    std::lock_guard<std::mutex> ak(s->admin);
    tw_ctx* c;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        Job* j = job_at(s, job);
        if (!j) return srv_fail_locked(s, TW_ERR_ARG, "no such job");
        if (!drain_job(s, lk, j, timeout_s))
            return srv_fail_locked(s, TW_ERR_TIMEOUT, "job has requests in flight");
        c = j->c;
        j->c = nullptr;
    }
    tw_ctx_destroy(c);
    return TW_OK;
}

int tw_server_job_cancel(tw_server* s, int32_t job, double timeout_s) {
    if (!s) return TW_ERR_ARG;
    std::lock_guard<std::mutex> ak(s->admin);
    tw_ctx* c;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        Job* j = job_at(s, job);
        if (!j) return srv_fail_locked(s, TW_ERR_ARG, "no such job");
        j->cancelling = true;
        // the job's requests still in the queue complete now, cancelled
        const auto now = Clock::now();
        for (auto it = s->queue.begin(); it != s->queue.end();) {
            Req* q = *it;
            if (q->job != job) {
                ++it;
                continue;
            }
            q->status = TW_ERR_CANCELLED;
            q->error = "job cancelled";
            q->t_done = now;
            q->done = true;
            j->pending -= 1;
            it = s->queue.erase(it);
        }
        s->cv.notify_all();
        // the batches already on a lane finish
        if (!drain_job(s, lk, j, timeout_s)) {
            j->cancelling = false;
            return srv_fail_locked(s, TW_ERR_TIMEOUT, "job has batches in flight");
        }
        c = j->c;
        j->c = nullptr;
        j->cancelling = false;
    }
    tw_ctx_destroy(c);
    return TW_OK;
}

int tw_server_submit(tw_server* s, int32_t job, const tw_request* req, uint64_t* ticket) {
    if (!s || !req || !ticket) return TW_ERR_ARG;
    const tw_request& r = *req;
    if (r.n < 0 || r.n > kMaxRequestItems) return srv_fail(s, TW_ERR_ARG, "bad request size");
    switch (r.kind) {
    case TW_REQ_POINTS:
    case TW_REQ_FACES:
        if (r.n > 0 && (!r.in0 || !r.out0)) return srv_fail(s, TW_ERR_ARG, "missing buffers");
        if (r.n > kMaxBatchQueries) return srv_fail(s, TW_ERR_TOO_LARGE, "request above batch cap");
        break;
    case TW_REQ_AMIPS:
        if (r.n > 0 && !r.in0) return srv_fail(s, TW_ERR_ARG, "missing buffers");
        break;
    case TW_REQ_SMOOTH: {
        if (r.n == 0) break;
        if (!r.in0 || !r.in1 || !r.in3 || !r.out0 || !r.out1)
            return srv_fail(s, TW_ERR_ARG, "missing buffers");
        if (r.in4 && !r.in2) return srv_fail(s, TW_ERR_ARG, "surface stars need face_flags");
        if (r.n > INT32_MAX - 1) return srv_fail(s, TW_ERR_TOO_LARGE, "too many stars");
        const int32_t* off = (const int32_t*)r.in0;
        if (off[0] != 0) return srv_fail(s, TW_ERR_ARG, "star offsets must start at 0");
        for (int64_t i = 0; i < r.n; ++i)
            if (off[i + 1] < off[i]) return srv_fail(s, TW_ERR_ARG, "star offsets decrease");
        if (r.in4) {
            const uint8_t* k = (const uint8_t*)r.in4;
            for (int64_t i = 0; i < r.n; ++i)
                if (k[i] > TW_STAR_BOUNDARY) return srv_fail(s, TW_ERR_ARG, "unknown star kind");
        }
        break;
    }
    default:
        return srv_fail(s, TW_ERR_ARG, "unknown request kind");
    }
    std::lock_guard<std::mutex> lk(s->mu);
    Job* j = job_at(s, job);
    if (!j) {
        s->last_error = "no such job";
        return TW_ERR_ARG;
    }
    if (j->cancelling) {
        s->last_error = "job is being cancelled";
        return TW_ERR_CANCELLED;
    }
    if (r.kind == TW_REQ_SMOOTH && r.n > 0) {
        if (!j->c->vx) {
            s->last_error = "job has no resident mesh";
            return TW_ERR_NO_MESH;
        }
        if (r.in4) {
            const uint8_t* k = (const uint8_t*)r.in4;
            bool bnd = false;
            for (int64_t i = 0; i < r.n && !bnd; ++i) bnd = k[i] == TW_STAR_BOUNDARY;
            if (bnd && j->c->surf[TW_SURFACE_BOUNDARY].nf == 0) {
                s->last_error = "no boundary surface for this job";
                return TW_ERR_NO_SURFACE;
            }
        }
    }
    Req* q = new Req();
    q->ticket = s->next_ticket++;
    q->job = job;
    q->r = r;
    q->t_submit = Clock::now();
    j->pending += 1;
    if (r.n == 0) {
        q->done = true;
        q->t_done = q->t_submit;
        j->pending -= 1;
    } else {
        s->queue.push_back(q);
    }
    s->reqs[q->ticket] = q;
    *ticket = q->ticket;
    s->cv.notify_all();
    return TW_OK;
}

int tw_server_wait(tw_server* s, uint64_t ticket, double timeout_s, double* latency_ms) {
    if (!s) return TW_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) {
        s->last_error = "unknown ticket";
        return TW_ERR_ARG;
    }
    Req* q = it->second;
    if (!s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return q->done; }))
        return TW_ERR_TIMEOUT;
    const int st = q->status;
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(q->t_done - q->t_submit).count();
    if (st != TW_OK) s->last_error = q->error;
    s->reqs.erase(it);
    delete q;
    return st;
}

int tw_server_get_stats(tw_server* s, tw_server_stats* out) {
    if (!s || !out) return TW_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    uint64_t open = 0;
    for (auto& j : s->jobs) open += j->c ? 1 : 0;
    out->jobs_open = open;
    out->bytes_used = jobs_bytes(s) + lanes_bytes(s);
    out->budget = s->budget;
    return TW_OK;
}

}  // extern "C"
