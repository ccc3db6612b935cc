// Serving loop: continuous batching of render requests over resident scenes.
//
// The reference renders one scene per GLUT frame callback (display(), main.cpp:1077-1368) with no
// request queue. Here a host thread runs steps: every step (1) admits queued requests while their
// device memory fits the server's HBM budget, (2) generates the current stage's rays of every in-flight
// request (primary rays, or one bounce's shadow + reflection rays), (3) traces all of them in ONE
// batched call (segmented hash/compress/sort/decompress, one persistent fused traversal + intersection
// launch), (4) resolves hits and advances each request; finished requests leave and new ones join
// between steps. Steps are enqueued without waiting for the GPU (at most two outstanding): the host
// admits and prepares the next step while the current one runs, and retires steps in order as their
// events complete. Ray state and results stay on the device until rsh_server_wait
// copies them out. A request's results do not depend on what else is in the batch: its rays form their
// own key segment, sort stably within it, and pack into work units of their own.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "engine.h"

using namespace rsh;

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    uint64_t id = 0;
    rsh_request r{};
    int32_t status = RSH_OK;
    double submit_ms = 0, start_ms = 0, finish_ms = 0;
    uint64_t rays = 0;
    bool done = false, cancelled = false, collected = false;
    uint32_t stage = 0;  // next stage to enqueue: 0 = primary; 1 + b = bounce b
    uint32_t pending = 0;     // enqueued steps not yet retired
    uint32_t stage_done = 0;  // stages whose step has retired
    size_t bytes = 0;
    // device buffers
    void* buf = nullptr;
    rsh_ray* prim_rays = nullptr;
    uint32_t* prim_pix = nullptr;
    unsigned long long* prim_hits = nullptr;
    float4* spos = nullptr;
    float4* snrm = nullptr;
    rsh_ray* srays = nullptr;
    rsh_ray* rrays[2] = {nullptr, nullptr};
    unsigned long long* hits = nullptr;  // depth x npix
    uint32_t* flags = nullptr;           // depth x npix x L
};

// A request's device buffers: one allocation, regions back to back, each starting on a 256-byte boundary.
// Returns the bytes the layout needs; with `q` and `base` set it also points q's buffers into `base`. The
// admission budget and the allocation both come from here, so the regions always fit.
size_t request_layout(const rsh_request& r, Req* q = nullptr, char* base = nullptr) {
    const size_t npix = (size_t)r.width * r.height;
    const size_t np = (size_t)((r.width + 7) / 8) * ((r.height + 7) / 8) * 64;
    const size_t L = r.light_count;
    size_t off = 0;
    auto take = [&](size_t n) {
        char* x = base ? base + off : nullptr;
        off += (n + 255) & ~size_t(255);
        return x;
    };
    char* prim_rays = take(np * 32);
    char* prim_pix = take(np * 4);
    char* prim_hits = take(np * 8);
    char* spos = take(npix * 16);
    char* snrm = take(npix * 16);
    char* srays = take(npix * L * 32);
    char* rrays0 = take(npix * 32);
    char* rrays1 = take(npix * 32);
    char* hits = take(npix * 8 * r.depth);
    char* flags = take(npix * L * 4 * r.depth);
    if (q && base) {
        q->prim_rays = reinterpret_cast<rsh_ray*>(prim_rays);
        q->prim_pix = reinterpret_cast<uint32_t*>(prim_pix);
        q->prim_hits = reinterpret_cast<unsigned long long*>(prim_hits);
        q->spos = reinterpret_cast<float4*>(spos);
        q->snrm = reinterpret_cast<float4*>(snrm);
        q->srays = reinterpret_cast<rsh_ray*>(srays);
        q->rrays[0] = reinterpret_cast<rsh_ray*>(rrays0);
        q->rrays[1] = reinterpret_cast<rsh_ray*>(rrays1);
        q->hits = reinterpret_cast<unsigned long long*>(hits);
        q->flags = reinterpret_cast<uint32_t*>(flags);
    }
    return off;
}

size_t request_bytes(const rsh_request& r) { return (request_layout(r) + 4095) & ~size_t(4095); }

}  // namespace

struct rsh_server {
    rsh_ctx* ctx = nullptr;
    std::vector<const rsh_scene*> scenes;
    uint64_t budget = 0;
    uint32_t max_inflight = 64;
    // rays one step may generate (primary pixels, or pixels x (lights + 1) for a bounce), the oldest
    // in-flight requests first; 0: every in-flight request each step (measured best up to saturation)
    uint64_t step_rays = 0;
    cudaStream_t stream = nullptr;
    // request buffers come from the server's own stream-ordered pool, allocated and freed on its stream:
    // a finished request's memory goes back without a device-wide synchronisation (cudaFree would stall
    // every step in flight), and the pool keeps it for the next request instead of returning it
    cudaMemPool_t pool = nullptr;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> queue;
    std::vector<Req*> inflight;
    std::map<uint64_t, Req*> all;
    uint64_t next_id = 1;
    bool stop = false;
    uint64_t completed = 0, steps = 0, peak_inflight = 0, bytes_in_use = 0, peak_bytes = 0;
    rsh_status fatal = RSH_OK;
    // steps enqueued on the stream and not yet retired (oldest first); each owns a pinned readback slot
    struct Step {
        cudaEvent_t done = nullptr;
        std::vector<Req*> act;       // requests with a stage in this step
        std::vector<size_t> seg_at;  // their first segment
        uint32_t* pinned = nullptr;  // segment counts, then the device error word
        size_t cap = 0;
    };
    std::deque<Step> steps_q;
    std::vector<Step> free_steps;  // retired records (event and pinned slot kept for reuse)
};

namespace {

rsh_status alloc_request(rsh_server* s, Req* q) {
    void* p = nullptr;
    // q->bytes = request_bytes(q->r) >= request_layout(q->r)
    RSH_CUDA(cudaMallocFromPoolAsync(&p, q->bytes, s->pool, s->stream));
    q->buf = p;
    request_layout(q->r, q, static_cast<char*>(p));
    return RSH_OK;
}

// The request's steps have all retired (or never ran): its buffer goes back to the pool in stream order.
void free_request(rsh_server* s, Req* q) {
    if (q->buf) {
        cudaFreeAsync(q->buf, s->stream);
        q->buf = nullptr;
        s->bytes_in_use -= q->bytes;
    }
}

// One step, enqueued without waiting (server thread, no lock held): generate the current stage's rays of
// every request in `act`, trace them all in one batched call, resolve the hits into the next surfaces,
// copy the segment counts and the device error word to the step's pinned slot and record its event.
// The host goes on admitting and enqueueing the next step while this one runs (at most kDepth steps are
// outstanding); steps retire in order when their events complete.
constexpr size_t kDepth = 2;

rsh_status enqueue_step(rsh_server* s, rsh_server::Step& rec) {
    cudaStream_t st = s->stream;
    std::vector<rsh_batch_segment> segs;
    segs.reserve(rec.act.size() * 2);
    rec.seg_at.clear();
    for (Req* q : rec.act) {
        const rsh_request& r = q->r;
        const rsh_scene* sc = s->scenes[r.scene_index];
        const uint32_t W = r.width, H = r.height, npix = W * H, L = r.light_count;
        rec.seg_at.push_back(segs.size());
        if (q->stage == 0) {
            CameraP cp;
            for (int i = 0; i < 3; ++i) {
                cp.eye[i] = r.camera.eye[i];
                cp.dir[i] = r.camera.direction[i];
                cp.right[i] = r.camera.right[i];
                cp.up[i] = r.camera.up[i];
            }
            RSH_CUDA(launch_raygen_primary(cp, W, H, q->prim_rays, q->prim_pix, st));
            const uint32_t np = ((W + 7) / 8) * ((H + 7) / 8) * 64;
            segs.push_back(rsh_batch_segment{sc, q->prim_rays, np, 0, reinterpret_cast<uint64_t*>(q->prim_hits),
                                             nullptr});
        } else {
            const uint32_t b = q->stage - 1;
            // the batched call keys every segment itself: the ray generators write no keys
            HashP hp_r;
            RSH_TRY(make_hash_params(sc, s->ctx->cfg, 0, hp_r));
            LightsP lp{};
            lp.count = L;
            lp.samples = 1;
            for (uint32_t l = 0; l < L; ++l)
                for (int i = 0; i < 3; ++i) lp.pos[l][i] = r.lights[l].position[i];
            RSH_CUDA(launch_raygen_shadow(q->spos, q->snrm, W, H, lp, s->ctx->cfg.epsilon, hp_r, q->srays, nullptr, st));
            const rsh_ray* prev = (b == 0) ? nullptr : q->rrays[(b - 1) & 1];
            rsh_ray* cur = q->rrays[b & 1];
            RSH_CUDA(launch_raygen_reflect(q->spos, q->snrm, prev, r.camera.eye, W, H, s->ctx->cfg.epsilon,
                                           s->ctx->cfg.reflect_jitter, s->ctx->cfg.seed, b, hp_r, cur, nullptr, st));
            segs.push_back(rsh_batch_segment{sc, q->srays, npix * L, 1, nullptr, q->flags + (size_t)b * npix * L});
            segs.push_back(rsh_batch_segment{sc, cur, npix, 0,
                                             reinterpret_cast<uint64_t*>(q->hits + (size_t)b * npix), nullptr});
        }
    }
    RSH_TRY(rsh_batch_trace(s->ctx, segs.data(), (uint32_t)segs.size(), st));
    if (rec.cap < segs.size() + 1) {
        if (rec.pinned) cudaFreeHost(rec.pinned);
        rec.pinned = nullptr;
        rec.cap = std::max<size_t>(segs.size() + 1, 256);
        RSH_CUDA(cudaMallocHost(&rec.pinned, 4 * rec.cap));
    }
    // rays traced per segment (after trimming): read when the step retires
    RSH_CUDA(cudaMemcpyAsync(rec.pinned, s->ctx->bufs["b_seg_cnt"].ptr, 4 * segs.size(), cudaMemcpyDeviceToHost,
                             st));
    // advance: resolve hits into the next surface
    for (Req* q : rec.act) {
        const rsh_request& r = q->r;
        const rsh_scene* sc = s->scenes[r.scene_index];
        const uint32_t W = r.width, H = r.height, npix = W * H;
        if (q->stage == 0) {
            const uint32_t np = ((W + 7) / 8) * ((H + 7) / 8) * 64;
            RSH_CUDA(launch_resolve(sc->pos, sc->nrm, sc->mat, q->prim_rays, q->prim_hits, q->prim_pix, np, q->spos,
                                    q->snrm, st));
        } else {
            const uint32_t b = q->stage - 1;
            RSH_CUDA(launch_resolve(sc->pos, sc->nrm, sc->mat, q->rrays[b & 1], q->hits + (size_t)b * npix, nullptr,
                                    npix, q->spos, q->snrm, st));
        }
    }
    // the device error word after this step (read, then cleared, in stream order)
    RSH_CUDA(cudaMemcpyAsync(rec.pinned + segs.size(), s->ctx->d_err, 4, cudaMemcpyDeviceToHost, st));
    RSH_CUDA(cudaMemsetAsync(s->ctx->d_err, 0, 4, st));
    if (!rec.done) RSH_CUDA(cudaEventCreateWithFlags(&rec.done, cudaEventDisableTiming));
    RSH_CUDA(cudaEventRecord(rec.done, st));
    return RSH_OK;
}

// Retires the oldest outstanding step once its event completed (waiting for it when `block`): adds each
// request's traced rays, finishes the requests whose last stage it was. Caller holds the lock; the wait
// itself runs unlocked. Returns false when nothing was retired.
bool retire_oldest(rsh_server* s, std::unique_lock<std::mutex>& lk, bool block) {
    if (s->steps_q.empty()) return false;
    rsh_server::Step& rec = s->steps_q.front();
    if (block) {
        lk.unlock();
        const cudaError_t e = cudaEventSynchronize(rec.done);
        lk.lock();
        if (e != cudaSuccess && s->fatal == RSH_OK) s->fatal = RSH_ERR_CUDA;
    } else if (cudaEventQuery(rec.done) == cudaErrorNotReady) {
        return false;
    }
    // the step's segments: each request's primary stage has one, a bounce two (steps retire in order, so a
    // request's stage in this step is its count of retired stages)
    size_t total_segs = 0;
    for (size_t k = 0; k < rec.act.size(); ++k) total_segs = rec.seg_at[k] + (rec.act[k]->stage_done == 0 ? 1 : 2);
    const uint32_t derr = rec.act.empty() ? 0u : rec.pinned[total_segs];
    for (size_t k = 0; k < rec.act.size(); ++k) {
        Req* q = rec.act[k];
        if (q->stage_done > 0) q->rays += (uint64_t)rec.pinned[rec.seg_at[k]] + rec.pinned[rec.seg_at[k] + 1];
        if (derr && q->status == RSH_OK) q->status = (derr & RSH_DEVERR_TIMEOUT) ? RSH_ERR_TIMEOUT : RSH_ERR_OVERFLOW;
        q->stage_done += 1;
        q->pending -= 1;
        if (q->pending == 0 && (q->stage_done > q->r.depth || q->cancelled || q->status != RSH_OK)) {
            q->done = true;
            q->finish_ms = now_ms();
            if (q->status == RSH_OK && q->cancelled) q->status = RSH_ERR_INVALID;
            if (q->status == RSH_OK) ++s->completed;
            s->inflight.erase(std::find(s->inflight.begin(), s->inflight.end(), q));
        }
    }
    if (derr && s->fatal == RSH_OK) s->fatal = (derr & RSH_DEVERR_TIMEOUT) ? RSH_ERR_TIMEOUT : RSH_ERR_OVERFLOW;
    rec.act.clear();
    s->free_steps.push_back(std::move(rec));
    s->steps_q.pop_front();
    s->cv_done.notify_all();
    return true;
}

void server_main(rsh_server* s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // retire what has finished, without waiting
        while (retire_oldest(s, lk, false)) {
        }
        // admission by HBM budget
        while (!s->queue.empty() && s->inflight.size() < s->max_inflight) {
            Req* q = s->queue.front();
            if (q->cancelled) {
                s->queue.pop_front();
                q->done = true;
                q->status = RSH_ERR_INVALID;
                q->finish_ms = now_ms();
                s->cv_done.notify_all();
                continue;
            }
            if (s->bytes_in_use + q->bytes > s->budget && !s->inflight.empty()) break;
            if (q->bytes > s->budget) {  // can never fit
                s->queue.pop_front();
                q->done = true;
                q->status = RSH_ERR_OOM;
                q->finish_ms = now_ms();
                s->cv_done.notify_all();
                continue;
            }
            s->queue.pop_front();
            s->bytes_in_use += q->bytes;
            if (alloc_request(s, q) != RSH_OK) {
                s->bytes_in_use -= q->bytes;
                q->done = true;
                q->status = RSH_ERR_OOM;
                q->finish_ms = now_ms();
                s->cv_done.notify_all();
                continue;
            }
            q->start_ms = now_ms();
            s->inflight.push_back(q);
        }
        s->peak_inflight = std::max<uint64_t>(s->peak_inflight, s->inflight.size());
        s->peak_bytes = std::max(s->peak_bytes, s->bytes_in_use);
        // cancelled in-flight requests with no step outstanding leave now; the others take no new stage
        for (auto it = s->inflight.begin(); it != s->inflight.end();) {
            Req* q = *it;
            if (q->cancelled && q->pending == 0) {
                free_request(s, q);
                q->done = true;
                q->status = RSH_ERR_INVALID;
                q->finish_ms = now_ms();
                it = s->inflight.erase(it);
                s->cv_done.notify_all();
            } else {
                ++it;
            }
        }
        // the requests with a stage left to enqueue, oldest first, up to the step's ray budget (at least one)
        std::vector<Req*> act;
        uint64_t step_rays = 0;
        for (Req* q : s->inflight) {
            if (q->cancelled || q->status != RSH_OK || q->stage > q->r.depth) continue;
            const uint64_t npix = (uint64_t)q->r.width * q->r.height;
            const uint64_t rays = q->stage == 0 ? npix : npix * (q->r.light_count + 1u);
            if (!act.empty() && s->step_rays && step_rays + rays > s->step_rays) break;
            step_rays += rays;
            act.push_back(q);
        }
        if (act.empty() || s->steps_q.size() >= kDepth) {
            if (!s->steps_q.empty()) {  // the GPU is busy: wait for its oldest step
                retire_oldest(s, lk, true);
                continue;
            }
            if (s->stop && s->queue.empty()) return;
            s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
            if (s->stop && s->queue.empty() && s->inflight.empty()) return;
            continue;
        }
        rsh_server::Step rec;
        if (!s->free_steps.empty()) {
            rec = std::move(s->free_steps.back());
            s->free_steps.pop_back();
        }
        rec.act = act;
        for (Req* q : act) q->pending += 1;
        lk.unlock();
        const rsh_status st = enqueue_step(s, rec);
        lk.lock();
        ++s->steps;
        if (st != RSH_OK) {
            // nothing of this step reached the GPU in a usable state: fail its requests once idle
            for (Req* q : act) {
                q->status = st;
                q->pending -= 1;
            }
            if (s->fatal == RSH_OK) s->fatal = st;
            lk.unlock();
            cudaStreamSynchronize(s->stream);
            lk.lock();
            for (Req* q : act) {
                if (q->pending == 0 && !q->done) {
                    q->done = true;
                    q->finish_ms = now_ms();
                    s->inflight.erase(std::find(s->inflight.begin(), s->inflight.end(), q));
                }
            }
            rec.act.clear();
            s->free_steps.push_back(std::move(rec));
            s->cv_done.notify_all();
            continue;
        }
        for (Req* q : act) q->stage += 1;
        s->steps_q.push_back(std::move(rec));
    }
}

}  // namespace

extern "C" {

rsh_status rsh_server_create(rsh_ctx* ctx, const rsh_scene* const* scenes, uint32_t scene_count, uint64_t hbm_budget,
                             uint32_t max_inflight, rsh_server** out) {
    if (!ctx || !scenes || !scene_count || !out) return RSH_ERR_INVALID;
    rsh_server* s = new rsh_server();
    s->ctx = ctx;
    s->scenes.assign(scenes, scenes + scene_count);
    s->budget = hbm_budget ? hbm_budget : (8ull << 30);
    s->max_inflight = max_inflight ? max_inflight : 64;
    if (2 * s->max_inflight > 1024) s->max_inflight = 512;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return cuda_status(e, "rsh_server_create");
    }
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = ~0ull;  // never trim the pool below what it holds: the budget bounds it
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e != cudaSuccess) {
        if (s->pool) cudaMemPoolDestroy(s->pool);
        cudaStreamDestroy(s->stream);
        delete s;
        return cuda_status(e, "rsh_server_create: memory pool");
    }
    s->th = std::thread(server_main, s);
    *out = s;
    return RSH_OK;
}

static bool request_fields_ok(const rsh_request* req) {
    return req && req->width != 0 && req->height != 0 && req->depth >= 1 && req->depth <= 4 &&
           req->light_count >= 1 && req->light_count <= 8 &&
           (uint64_t)req->width * req->height * req->light_count < (1ull << 31);
}

rsh_status rsh_server_request_bytes(const rsh_request* req, uint64_t* bytes) {
    if (!bytes || !request_fields_ok(req)) return RSH_ERR_INVALID;
    *bytes = request_bytes(*req);
    return RSH_OK;
}

rsh_status rsh_server_submit(rsh_server* s, const rsh_request* req, uint64_t* id_out) {
    if (!s || !request_fields_ok(req) || req->scene_index >= s->scenes.size()) return RSH_ERR_INVALID;
    Req* q = new Req();
    q->r = *req;
    q->bytes = request_bytes(*req);
    q->submit_ms = now_ms();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        q->id = s->next_id++;
        s->all[q->id] = q;
        s->queue.push_back(q);
    }
    s->cv_work.notify_one();
    if (id_out) *id_out = q->id;
    return RSH_OK;
}

rsh_status rsh_server_wait(rsh_server* s, uint64_t id, uint32_t timeout_ms, rsh_request_result* result,
                           uint64_t* hits_host, uint32_t* flags_host) {
    if (!s) return RSH_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return RSH_ERR_INVALID;
    Req* q = it->second;
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return q->done; })) {
        set_error("request not finished");
        return RSH_ERR_TIMEOUT;
    }
    if (result) {
        result->id = q->id;
        result->status = q->status;
        result->submit_ms = q->submit_ms;
        result->start_ms = q->start_ms;
        result->finish_ms = q->finish_ms;
        result->rays = q->rays;
    }
    const rsh_request& r = q->r;
    const size_t npix = (size_t)r.width * r.height;
    if (q->buf && q->status == RSH_OK) {
        if (hits_host) RSH_CUDA(cudaMemcpy(hits_host, q->hits, npix * 8 * r.depth, cudaMemcpyDeviceToHost));
        if (flags_host)
            RSH_CUDA(cudaMemcpy(flags_host, q->flags, npix * r.light_count * 4 * r.depth, cudaMemcpyDeviceToHost));
    }
    free_request(s, q);
    s->all.erase(it);
    const int32_t st = q->status;
    delete q;
    s->cv_work.notify_one();
    return (rsh_status)st;
}

rsh_status rsh_server_cancel(rsh_server* s, uint64_t id) {
    if (!s) return RSH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return RSH_ERR_INVALID;
    it->second->cancelled = true;
    s->cv_work.notify_one();
    return RSH_OK;
}

rsh_status rsh_server_set_step_rays(rsh_server* s, uint64_t rays) {
    if (!s) return RSH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->step_rays = rays;
    return RSH_OK;
}

rsh_status rsh_server_stats(rsh_server* s, uint64_t* completed, uint64_t* steps, uint64_t* peak_inflight,
                            uint64_t* peak_bytes) {
    if (!s) return RSH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (completed) *completed = s->completed;
    if (steps) *steps = s->steps;
    if (peak_inflight) *peak_inflight = s->peak_inflight;
    if (peak_bytes) *peak_bytes = s->peak_bytes;
    return s->fatal;
}

rsh_status rsh_server_destroy(rsh_server* s) {
    if (!s) return RSH_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Req* q : s->queue) q->cancelled = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();
    for (auto& kv : s->all) {
        free_request(s, kv.second);
        delete kv.second;
    }
    cudaStreamSynchronize(s->stream);
    for (auto* list : {&s->free_steps}) {
        for (auto& rec : *list) {
            if (rec.done) cudaEventDestroy(rec.done);
            if (rec.pinned) cudaFreeHost(rec.pinned);
        }
    }
    for (auto& rec : s->steps_q) {
        if (rec.done) cudaEventDestroy(rec.done);
        if (rec.pinned) cudaFreeHost(rec.pinned);
    }
    cudaStreamSynchronize(s->stream);
    cudaMemPoolDestroy(s->pool);
    cudaStreamDestroy(s->stream);
    delete s;
    return RSH_OK;
}

}  // extern "C"
