// Serving loop of the compute stage (config 4): continuous batching of
// per-session frame requests.  No counterpart in the reference, whose single
// window renders one view per frame (main.cpp:172-194); each request here is
// one reference frame -- checkerboard raymarch + reprojection of a session's
// previous frame -- for one of many sessions.
//
//   * A session owns its resident state on the device: the two raw frames the
//     reprojection ping-pongs between (Renderer.cpp:131-136, 191), the god-ray
//     mask and the previous camera (main.cpp:185-186).  Sessions are admitted
//     while their state fits the HBM budget.
//   * Requests queue in arrival order.  A worker thread forms a batch from
//     every queued request whose session has no frame in flight (a session's
//     frame N+1 reprojects frame N), up to max_batch, and launches it with
//     mt_render_batch (a batch of one with mt_render, which skips the batch's
//     tables).  Up to `streams` batches are in flight at once: requests
//     that arrive while a batch runs join the next one, which overlaps on the
//     device.  Completion is stamped by a host function queued behind the
//     batch on its stream.
//   * Every result equals the same request rendered alone (the batched launch
//     is exact per pixel); tests check it.
//
// Threading: the server is the only user of its context while it runs.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/meteoros.h"

namespace mt {
int ctx_device(const mt_ctx* ctx);  // mt_capi.cu
}

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Session {
    int64_t id = 0;
    int w = 0, h = 0;
    mt_params params{};
    mt_camera_ubo last_cam{};
    bool has_prev = false;
    bool busy = false;
    int parity = 0;
    float* raw[2] = {nullptr, nullptr};
    float* mask = nullptr;
    uint64_t bytes = 0;
};

struct Request {
    uint64_t id = 0;
    int64_t session = 0;
    mt_camera_ubo cam{};
    mt_time_ubo time{};
    double submit_s = 0, start_s = 0, done_s = 0;
    int32_t batch = 0;
    int32_t status = MT_OK;
    bool done = false;
};

struct Batch;

}  // namespace

struct mt_server {
    mt_ctx* ctx = nullptr;
    int device = 0;
    mt_server_config cfg{};
    mt_tuning saved{};  // the context's tuning before the server changed it
    bool restore = false;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::unordered_map<int64_t, Session> sessions;
    std::unordered_map<uint64_t, Request> requests;
    std::deque<uint64_t> pending;
    int inflight = 0;
    int next_stream = 0;
    cudaStream_t streams[2] = {nullptr, nullptr};
    std::thread worker;
    bool stop = false;
    uint64_t used_bytes = 0;
    int64_t next_session = 1;
    uint64_t next_request = 1;
    std::string err;
};

namespace {

struct Batch {
    mt_server* srv;
    std::vector<uint64_t> reqs;
};

// Runs on a CUDA driver thread once the batch's work has finished: no CUDA
// calls here, only bookkeeping.
void CUDART_CB on_batch_done(void* data) {
    Batch* b = static_cast<Batch*>(data);
    mt_server* s = b->srv;
    const double t = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (uint64_t id : b->reqs) {
            auto it = s->requests.find(id);
            if (it == s->requests.end()) continue;
            Request& r = it->second;
            r.done_s = t;
            r.done = true;
            auto ss = s->sessions.find(r.session);
            if (ss != s->sessions.end()) {
                Session& se = ss->second;
                se.busy = false;
                if (r.status == MT_OK) {
                    se.parity ^= 1;
                    se.has_prev = true;
                    se.last_cam = r.cam;
                }
            }
        }
        s->inflight--;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    delete b;
}

bool can_form_batch(mt_server* s) {
    if (s->pending.empty() || s->inflight >= s->cfg.streams) return false;
    for (uint64_t id : s->pending) {
        auto rq = s->requests.find(id);
        if (rq == s->requests.end()) return true;  // dropped by the next pass
        auto it = s->sessions.find(rq->second.session);
        if (it == s->sessions.end() || !it->second.busy) return true;
    }
    return false;
}

void worker_main(mt_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        s->cv_work.wait(lk, [&] { return s->stop || can_form_batch(s); });
        if (s->stop) break;
        // Form a batch: queued requests in arrival order whose session is idle.
        std::vector<uint64_t> take;
        std::vector<mt_view> views;
        std::deque<uint64_t> keep;
        const int max_batch = s->cfg.per_request ? 1 : std::max(1, s->cfg.max_batch);
        for (uint64_t id : s->pending) {
            auto rq = s->requests.find(id);
            if (rq == s->requests.end()) continue;
            Request& r = rq->second;
            auto it = s->sessions.find(r.session);
            if (it == s->sessions.end()) {  // session closed: fail the request
                r.status = MT_ERR_INVALID_ARG;
                r.done = true;
                r.done_s = now_s();
                continue;
            }
            Session& se = it->second;
            if ((int)take.size() >= max_batch || se.busy) {
                keep.push_back(id);
                continue;
            }
            se.busy = true;
            take.push_back(id);
            mt_view v;
            std::memset(&v, 0, sizeof(v));
            v.camera = r.cam;
            v.camera_old = se.has_prev ? se.last_cam : r.cam;
            v.time = r.time;
            v.params = se.params;
            v.prev_rgba = se.has_prev ? se.raw[se.parity ^ 1] : nullptr;
            v.cur_rgba = se.raw[se.parity];
            v.godray_mask = se.mask;
            v.width = se.w;
            v.height = se.h;
            // a session's first frame has nothing to reproject: every pixel is marched
            v.flags = (se.has_prev ? MT_RENDER_CHECKERBOARD : MT_RENDER_FULL) | MT_RENDER_COUNT;
            views.push_back(v);
        }
        s->pending.swap(keep);
        s->cv_done.notify_all();
        if (take.empty()) continue;
        const double t_start = now_s();
        for (uint64_t id : take) {
            Request& r = s->requests[id];
            r.start_s = t_start;
            r.batch = (int32_t)take.size();
        }
        s->inflight++;
        cudaStream_t stream = s->streams[s->next_stream];
        s->next_stream = (s->next_stream + 1) % std::max(1, s->cfg.streams);
        lk.unlock();
        mt_status st;
        // A batch of one takes the direct launch: the same frame as the batched
        // launch (equal per pixel), without building a view table and tile list.
        if (s->cfg.per_request || views.size() == 1) {
            const mt_view& v = views[0];
            st = mt_render(s->ctx, &v.camera, &v.camera_old, &v.time, &v.params, v.prev_rgba, v.cur_rgba,
                           v.godray_mask, v.width, v.height, v.flags, stream);
        } else {
            st = mt_render_batch(s->ctx, views.data(), (int)views.size(), stream);
        }
        Batch* b = new Batch{s, take};
        cudaError_t e = cudaSuccess;
        if (st == MT_OK) e = cudaLaunchHostFunc(stream, on_batch_done, b);
        lk.lock();
        if (st != MT_OK || e != cudaSuccess) {
            s->err = st != MT_OK ? mt_last_error(s->ctx) : cudaGetErrorString(e);
            for (uint64_t id : take) s->requests[id].status = st != MT_OK ? st : MT_ERR_CUDA;
            lk.unlock();
            on_batch_done(b);  // marks the requests done (failed)
            lk.lock();
        }
    }
}

// Wait predicate of the calls that wait for a session's frame in flight.  The
// session is looked up by key at every wake-up, never through an iterator kept
// across the wait: the lock is released while waiting, and another caller may
// close the session or insert into the map (a rehash invalidates iterators).
bool session_idle_or_gone(mt_server* s, int64_t session) {
    auto j = s->sessions.find(session);
    return j == s->sessions.end() || !j->second.busy;
}

mt_status sfail(mt_server* s, mt_status st, const char* msg) {
    if (s) s->err = msg;
    return st;
}

}  // namespace

extern "C" {

MT_API double mt_server_clock(void) { return now_s(); }

MT_API mt_status mt_server_create(mt_ctx* ctx, const mt_server_config* cfg, mt_server** out) {
    if (!ctx || !cfg || !out) return MT_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->max_batch < 1 || cfg->streams < 1 || cfg->streams > 2) return MT_ERR_INVALID_ARG;
    mt_server* s = new (std::nothrow) mt_server();
    if (!s) return MT_ERR_OUT_OF_MEMORY;
    s->ctx = ctx;
    s->device = mt::ctx_device(ctx);
    s->cfg = *cfg;
    if (cudaSetDevice(s->device) != cudaSuccess) {
        delete s;
        return MT_ERR_CUDA;
    }
    for (int k = 0; k < s->cfg.streams; ++k)
        if (cudaStreamCreateWithFlags(&s->streams[k], cudaStreamNonBlocking) != cudaSuccess) {
            mt_server_destroy(s);
            return MT_ERR_CUDA;
        }
    mt_tuning t;
    mt_get_tuning(ctx, &t);
    s->saved = t;
    s->restore = true;
    if (cfg->batch_lanes) t.batch_lanes = cfg->batch_lanes;
    t.batch_direct = cfg->use_graph ? 0 : 1;
    if (mt_set_tuning(ctx, &t) != MT_OK) {
        mt_server_destroy(s);
        return MT_ERR_INVALID_ARG;
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return MT_OK;
}

MT_API void mt_server_destroy(mt_server* s) {
    if (!s) return;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        // bounded drain of the batches in flight (each is milliseconds of work)
        s->cv_done.wait_for(lk, std::chrono::seconds(30), [&] { return s->inflight == 0; });
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (cudaStream_t st : s->streams)
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    if (s->restore) mt_set_tuning(s->ctx, &s->saved);
    for (auto& kv : s->sessions) {
        cudaFree(kv.second.raw[0]);
        cudaFree(kv.second.raw[1]);
        cudaFree(kv.second.mask);
    }
    delete s;
}

MT_API const char* mt_server_last_error(const mt_server* s) { return s ? s->err.c_str() : ""; }

MT_API mt_status mt_server_open_session(mt_server* s, int width, int height, const mt_params* params,
                                        int64_t* session) {
    if (!s || !params || !session) return MT_ERR_INVALID_ARG;
    if (width < 1 || height < 1 || width > MT_MAX_DIM || height > MT_MAX_DIM)
        return sfail(s, MT_ERR_INVALID_ARG, "bad session size");
    const uint64_t px = (uint64_t)width * (uint64_t)height;
    const uint64_t bytes = px * (2 * 16 + 4);
    {
        // reserve the budget; allocation happens outside the lock (a CUDA
        // call that waits for the device must not hold the lock the
        // completion callbacks take)
        std::unique_lock<std::mutex> lk(s->mu);
        if (bytes > s->cfg.hbm_budget_bytes)
            return sfail(s, MT_ERR_BUDGET, "session is larger than the HBM budget");
        // admitted when closing sessions free enough of the budget, within the wait
        const auto fits = [&] { return s->used_bytes + bytes <= s->cfg.hbm_budget_bytes; };
        if (!fits() && !(s->cfg.admission_wait_ms > 0 &&
                         s->cv_done.wait_for(lk, std::chrono::milliseconds(s->cfg.admission_wait_ms), fits)))
            return sfail(s, MT_ERR_BUDGET, "session does not fit the HBM budget");
        s->used_bytes += bytes;
    }
    Session se;
    se.w = width;
    se.h = height;
    se.params = *params;
    se.bytes = bytes;
    cudaSetDevice(s->device);
    if (cudaMalloc((void**)&se.raw[0], px * 16) != cudaSuccess ||
        cudaMalloc((void**)&se.raw[1], px * 16) != cudaSuccess || cudaMalloc((void**)&se.mask, px * 4) != cudaSuccess) {
        cudaFree(se.raw[0]);
        cudaFree(se.raw[1]);
        cudaFree(se.mask);
        cudaGetLastError();
        std::lock_guard<std::mutex> lk(s->mu);
        s->used_bytes -= bytes;
        return sfail(s, MT_ERR_OUT_OF_MEMORY, "cudaMalloc of session state failed");
    }
    std::lock_guard<std::mutex> lk(s->mu);
    se.id = s->next_session++;
    *session = se.id;
    s->sessions.emplace(se.id, se);
    return MT_OK;
}

MT_API mt_status mt_server_close_session(mt_server* s, int64_t session) {
    if (!s) return MT_ERR_INVALID_ARG;
    Session se;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->sessions.find(session) == s->sessions.end()) return sfail(s, MT_ERR_INVALID_ARG, "unknown session");
        // wait (bounded) for the session's frame in flight, or for another
        // caller to close it meanwhile
        if (!s->cv_done.wait_for(lk, std::chrono::seconds(30), [&] { return session_idle_or_gone(s, session); }))
            return sfail(s, MT_ERR_TIMEOUT, "session still busy");
        auto it = s->sessions.find(session);
        if (it == s->sessions.end()) return sfail(s, MT_ERR_INVALID_ARG, "session closed meanwhile");
        se = it->second;
        s->sessions.erase(it);
    }
    s->cv_work.notify_all();  // its queued requests are failed by the worker
    cudaSetDevice(s->device);
    cudaFree(se.raw[0]);
    cudaFree(se.raw[1]);
    cudaFree(se.mask);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->used_bytes -= se.bytes;
    }
    s->cv_done.notify_all();  // budget freed: a waiting admission may proceed
    return MT_OK;
}

MT_API mt_status mt_server_submit(mt_server* s, int64_t session, const mt_camera_ubo* camera,
                                  const mt_time_ubo* time, uint64_t* request) {
    if (!s || !camera || !time) return MT_ERR_INVALID_ARG;
    if (time->frame_count_mod16 < 0 || time->frame_count_mod16 > 15)
        return sfail(s, MT_ERR_INVALID_ARG, "frame_count_mod16 outside 0..15");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->sessions.find(session) == s->sessions.end()) return sfail(s, MT_ERR_INVALID_ARG, "unknown session");
        Request r;
        r.id = s->next_request++;
        r.session = session;
        r.cam = *camera;
        r.time = *time;
        r.submit_s = now_s();
        s->requests.emplace(r.id, r);
        s->pending.push_back(r.id);
        if (request) *request = r.id;
    }
    s->cv_work.notify_one();
    return MT_OK;
}

MT_API mt_status mt_server_wait(mt_server* s, uint64_t request, int timeout_ms, mt_request_info* out) {
    if (!s) return MT_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->requests.find(request) == s->requests.end()) return sfail(s, MT_ERR_INVALID_ARG, "unknown request");
    // looked up again at every wake-up: another waiter may have taken the
    // request, and inserts may rehash the map (both invalidate iterators)
    const auto done_or_gone = [&] {
        auto j = s->requests.find(request);
        return j == s->requests.end() || j->second.done;
    };
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)), done_or_gone))
        return MT_ERR_TIMEOUT;
    auto it = s->requests.find(request);
    if (it == s->requests.end()) return sfail(s, MT_ERR_INVALID_ARG, "request taken by another waiter");
    const Request& r = it->second;
    if (out) {
        out->id = r.id;
        out->session = r.session;
        out->submit_s = r.submit_s;
        out->start_s = r.start_s;
        out->done_s = r.done_s;
        out->batch_size = r.batch;
        out->status = r.status;
    }
    const mt_status st = (mt_status)r.status;
    s->requests.erase(it);
    return st;
}

MT_API mt_status mt_server_read_frame(mt_server* s, int64_t session, float* host_rgba, float* host_mask) {
    if (!s) return MT_ERR_INVALID_ARG;
    const float* src_rgba = nullptr;
    const float* src_mask = nullptr;
    size_t px = 0;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->sessions.find(session) == s->sessions.end()) return sfail(s, MT_ERR_INVALID_ARG, "unknown session");
        if (!s->cv_done.wait_for(lk, std::chrono::seconds(30), [&] { return session_idle_or_gone(s, session); }))
            return sfail(s, MT_ERR_TIMEOUT, "session still busy");
        auto it = s->sessions.find(session);
        if (it == s->sessions.end()) return sfail(s, MT_ERR_INVALID_ARG, "session closed meanwhile");
        Session& se = it->second;
        if (!se.has_prev) return sfail(s, MT_ERR_NO_VOLUMES, "session has no frame yet");
        se.busy = true;  // no frame of the session starts while it is read
        src_rgba = se.raw[se.parity ^ 1];
        src_mask = se.mask;
        px = (size_t)se.w * (size_t)se.h;
    }
    cudaSetDevice(s->device);
    cudaError_t e = cudaSuccess;
    if (host_rgba) e = cudaMemcpy(host_rgba, src_rgba, px * 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && host_mask) e = cudaMemcpy(host_mask, src_mask, px * 4, cudaMemcpyDeviceToHost);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->sessions.find(session);
        if (it != s->sessions.end()) it->second.busy = false;
        if (e != cudaSuccess) s->err = std::string("read of the session frame failed: ") + cudaGetErrorString(e);
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    return e == cudaSuccess ? MT_OK : MT_ERR_CUDA;
}

MT_API mt_status mt_server_memory(mt_server* s, uint64_t* used_bytes, uint64_t* budget_bytes) {
    if (!s) return MT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (used_bytes) *used_bytes = s->used_bytes;
    if (budget_bytes) *budget_bytes = s->cfg.hbm_budget_bytes;
    return MT_OK;
}

}  // extern "C"
