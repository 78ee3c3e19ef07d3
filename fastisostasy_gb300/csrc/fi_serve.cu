// fi_serve.cu — continuous-batching solve server and batched ensembles.
//
// A request is one LV-ELVA solve: a domain (parameters, ice grid, padded
// rheology fields), a constant ice load and a horizon, advanced by
// isos_update calls every dtt.  Two kinds of host threads share the work:
//
//   workers   (kWorkers threads) admit queued requests as long as the
//             in-flight cap and free HBM (cudaMemGetInfo, less a reserve and
//             less the estimates of requests still being set up) allow, and
//             turn them into handles (fi_create + fields + init: host-side
//             set-up that must not stall the stepping); they also retire
//             finished requests: device status, w and z_bed on the ice grid,
//             handle freed, which makes room for the next admission.  The
//             footprint of each padded size is learnt from its first handle.
//   scheduler (one thread) steps: every running request keeps up to kDepth
//             updates queued on its own stream (fi_update_async: one captured
//             CUDA graph per update), so the updates of different requests
//             overlap on the GPU, and a request set up while others run joins
//             at the next round.
//
// A request's arithmetic does not depend on what else runs: every handle has
// its own buffers and stream and every reduction is deterministic, so a
// result is bit-identical alone and in a mix.
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fi_gpu.h"

namespace {

constexpr int kDepth = 2;     // updates queued ahead per running request
constexpr int kWorkers = 4;   // set-up / retire threads

struct Req {
    uint64_t id = 0;
    fi_params p;
    int nxi = 0, nyi = 0;
    double dx = 0, dy = 0;
    std::vector<double> z_bed, Href, H, D, eta, R;
    std::vector<uint8_t> mask;
    double t0 = 0, t_end = 0, dtt = 0, bsl = 0;
    // runtime
    fi_handle* h = nullptr;
    fi_bsl b;
    long long k = 0, nsteps = 0;   // updates issued / total
    double* dH = nullptr;          // the load on the device, handed to the first update
    int nout = 0, head = 0;
    int fail_rc = 0;               // stepping failed with this status
    std::atomic<bool> cancel{false};   // fi_serve_cancel: stop issuing, retire when idle
    cudaEvent_t ev[kDepth] = {nullptr, nullptr};
    int32_t pd[6] = {0, 0, 0, 0, 0, 0};
    size_t mem_key = 0;
    fi_request_info info;
    std::vector<double> w_out, zb_out;
};

}  // namespace

struct fi_server {
    int device = 0;
    int max_inflight = 1;
    size_t reserve = 0;
    size_t device_total = 0;           // bytes of device memory (admission bound)
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;        // wakes the scheduler
    std::condition_variable work_cv;   // wakes the workers
    std::condition_variable done_cv;   // wakes waiters
    std::deque<Req*> queue;            // submitted, not admitted
    std::deque<Req*> ready;            // set up, joining the scheduler
    std::deque<Req*> retiring;         // stepped to t_end (or failed), to be collected
    std::vector<Req*> active;          // scheduler thread only
    int inflight = 0;                  // admitted and not yet retired
    size_t pending_bytes = 0;          // footprint estimates of requests being set up
    std::unordered_map<uint64_t, Req*> all;
    std::map<size_t, size_t> footprint;   // padded cells * 2 + precision -> bytes
    uint64_t next_id = 1;
    bool stop = false;
    std::thread th;
    std::vector<std::thread> workers;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

void finish(fi_server* s, Req* r, int state, int status)
{
    if (state == 3 && !r->info.error[0]) {
        const char* m = r->h ? fi_last_error(r->h) : "";
        snprintf(r->info.error, sizeof(r->info.error), "%s", (m && m[0]) ? m : "solve failed");
    }
    if (r->h) {
        fi_destroy(r->h);
        r->h = nullptr;
    }
    for (auto& e : r->ev)
        if (e) { cudaEventDestroy(e); e = nullptr; }
    if (r->dH) {
        cudaFree(r->dH);
        r->dH = nullptr;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    r->info.state = state;
    r->info.status = status;
    r->info.t_done = s->now();
    // the inputs are no longer needed
    std::vector<double>().swap(r->z_bed);
    std::vector<double>().swap(r->Href);
    std::vector<double>().swap(r->H);
    std::vector<double>().swap(r->D);
    std::vector<double>().swap(r->eta);
    std::vector<double>().swap(r->R);
    std::vector<uint8_t>().swap(r->mask);
    s->done_cv.notify_all();
}

// Create, fill and initialise the handle of a request.
int start(fi_server* s, Req* r)
{
    size_t free0 = 0, total = 0;
    cudaMemGetInfo(&free0, &total);
    int rc = fi_create(&r->p, r->nxi, r->nyi, r->dx, r->dy, nullptr, &r->h);
    if (rc) return rc;
    rc = fi_set_fields(r->h, r->D.empty() ? nullptr : r->D.data(), r->eta.empty() ? nullptr : r->eta.data(),
                       r->R.empty() ? nullptr : r->R.data(), r->mask.empty() ? nullptr : r->mask.data());
    if (rc) return rc;
    memset(&r->b, 0, sizeof(r->b));
    r->b.method = 0;
    r->b.constant_ocean_surface = 1;
    r->b.bsl_init = r->b.bsl_now = r->bsl;
    r->b.A_ocean_pd = r->b.A_ocean_now = 3.625e14;
    if ((rc = fi_init_state(r->h, r->z_bed.data(), r->Href.data(), r->t0, &r->b))) return rc;
    const size_t hb = r->H.size() * sizeof(double);
    if (cudaMalloc(&r->dH, hb) != cudaSuccess) return FI_E_OOM;
    // On the handle's stream: a plain cudaMemcpy from pageable memory may
    // return before its DMA lands, and the handle's non-blocking stream, which
    // reads the load first thing in the first update, is not ordered after it.
    cudaStream_t hs = (cudaStream_t)fi_stream(r->h);
    if (cudaMemcpyAsync(r->dH, r->H.data(), hb, cudaMemcpyHostToDevice, hs) != cudaSuccess ||
        cudaStreamSynchronize(hs) != cudaSuccess)
        return FI_E_CUDA;
    for (auto& e : r->ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return FI_E_CUDA;
    size_t free1 = 0;
    cudaMemGetInfo(&free1, &total);
    if (free0 > free1) {
        std::lock_guard<std::mutex> lk(s->mu);
        size_t& f = s->footprint[r->mem_key];
        if (free0 - free1 > f) f = free0 - free1;
    }
    return FI_OK;
}

size_t estimate(fi_server* s, const Req* r)
{
    auto it = s->footprint.find(r->mem_key);
    if (it != s->footprint.end()) return it->second;
    // before the first handle of this size: about 100 doubles per padded cell
    // plus the (2n)^2 convolution spectra
    const size_t n = (size_t)r->pd[0] * r->pd[1];
    return n * 800 + 8 * n * 16;
}

// Called with s->mu held.
bool can_admit(fi_server* s, size_t* est)
{
    if (s->queue.empty() || s->inflight >= s->max_inflight) return false;
    *est = estimate(s, s->queue.front());
    if (s->inflight == 0) return true;   // an idle server always takes one
    size_t free_b = 0, total = 0;
    cudaMemGetInfo(&free_b, &total);
    return free_b >= s->pending_bytes + *est + s->reserve;
}

void collect(fi_server* s, Req* r)
{
    if (r->fail_rc == FI_E_CANCELLED || (r->cancel.load() && !r->fail_rc)) {
        // the request's stream is idle (no update in flight): drop the handle
        finish(s, r, 4, FI_E_CANCELLED);
        return;
    }
    if (r->fail_rc) {
        finish(s, r, 3, r->fail_rc);
        return;
    }
    int st = fi_synchronize(r->h);
    if (st == FI_OK && r->nsteps > 0) {
        // the model clock must have reached t_end: a request whose solve did
        // not advance is an error, never a result
        double sc[16];
        if ((st = fi_get_scalars(r->h, sc)) == FI_OK &&
            !(fabs(sc[0] - r->t_end) <= 1e-9 * fmax(1.0, fabs(r->t_end)))) {
            snprintf(r->info.error, sizeof(r->info.error), "model clock %.9g short of t_end %.9g (dt %.3g, %d steps)",
                     sc[0], r->t_end, sc[1], (int)sc[9]);
            st = FI_E_STATE;
        }
    }
    if (st == FI_OK) {
        const int nx = r->pd[0];
        std::vector<double> pad((size_t)r->pd[0] * r->pd[1]);
        r->w_out.resize((size_t)r->nxi * r->nyi);
        r->zb_out.resize((size_t)r->nxi * r->nyi);
        const int i0 = r->pd[2] - 1, j0 = r->pd[4] - 1;
        int rc = fi_get_field(r->h, FI_FIELD_W, pad.data());
        for (int j = 0; j < r->nyi && !rc; ++j)
            memcpy(&r->w_out[(size_t)j * r->nxi], &pad[(size_t)(j + j0) * nx + i0], r->nxi * sizeof(double));
        if (!rc) rc = fi_get_field(r->h, FI_FIELD_Z_BED, pad.data());
        for (int j = 0; j < r->nyi && !rc; ++j)
            memcpy(&r->zb_out[(size_t)j * r->nxi], &pad[(size_t)(j + j0) * nx + i0], r->nxi * sizeof(double));
        st = rc;
    }
    finish(s, r, st == FI_OK ? 2 : 3, st);
}

void worker(fi_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        if (!s->retiring.empty()) {
            Req* r = s->retiring.front();
            s->retiring.pop_front();
            lk.unlock();
            collect(s, r);
            lk.lock();
            s->inflight--;
            s->work_cv.notify_all();
            s->cv.notify_one();
            continue;
        }
        size_t est = 0;
        if (!s->queue.empty() && s->device_total &&
            estimate(s, s->queue.front()) + s->reserve > s->device_total) {
            // admission can never succeed: the request's estimated footprint
            // plus the reserve exceeds the device's memory
            Req* r = s->queue.front();
            s->queue.pop_front();
            snprintf(r->info.error, sizeof(r->info.error),
                     "needs about %.2f GB + reserve %.2f GB, device has %.2f GB",
                     estimate(s, r) / 1e9, s->reserve / 1e9, s->device_total / 1e9);
            lk.unlock();
            finish(s, r, 3, FI_E_OOM);
            lk.lock();
            continue;
        }
        if (can_admit(s, &est)) {
            Req* r = s->queue.front();
            s->queue.pop_front();
            s->inflight++;
            s->pending_bytes += est;
            r->info.state = 1;
            r->info.t_admit = s->now();
            lk.unlock();
            const int rc = start(s, r);
            if (rc) finish(s, r, 3, rc);
            lk.lock();
            s->pending_bytes -= est;
            if (rc) {
                s->inflight--;
                s->work_cv.notify_all();
            } else {
                s->ready.push_back(r);
            }
            s->cv.notify_one();
            continue;
        }
        if (s->stop && s->queue.empty() && s->retiring.empty() && s->inflight == 0) return;
        s->work_cv.wait(lk);
    }
}

void run(fi_server* s)
{
    cudaSetDevice(s->device);
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            while (!s->ready.empty()) {
                s->active.push_back(s->ready.front());
                s->ready.pop_front();
            }
            if (s->active.empty() && s->stop && s->queue.empty() && s->inflight == 0) return;
        }
        bool work = false;
        std::vector<Req*> out;
        for (size_t a = 0; a < s->active.size();) {
            Req* r = s->active[a];
            while (r->nout > 0 && cudaEventQuery(r->ev[r->head]) == cudaSuccess) {
                r->head = (r->head + 1) % kDepth;
                r->nout--;
                work = true;
            }
            int rc = FI_OK;
            const bool cancelled = r->cancel.load();
            while (!cancelled && r->nout < kDepth && r->k < r->nsteps) {
                // the same time sequence as a caller stepping by dtt, clipped at t_end
                double tn = r->t0 + (double)(r->k + 1) * r->dtt;
                if (r->k + 1 == r->nsteps || tn > r->t_end) tn = r->t_end;
                if ((rc = fi_update_async(r->h, r->k == 0 ? r->dH : nullptr, tn, &r->b))) break;
                cudaEventRecord(r->ev[(r->head + r->nout) % kDepth], (cudaStream_t)fi_stream(r->h));
                r->nout++;
                r->k++;
                work = true;
            }
            if (rc || (r->nout == 0 && (cancelled || r->k >= r->nsteps))) {
                r->fail_rc = rc ? rc : (cancelled ? FI_E_CANCELLED : 0);
                out.push_back(r);
                s->active.erase(s->active.begin() + a);
                work = true;
                continue;
            }
            ++a;
        }
        std::unique_lock<std::mutex> lk(s->mu);
        for (Req* r : s->active) r->info.updates = r->k;
        if (!out.empty()) {
            for (Req* r : out) {
                r->info.updates = r->k;
                s->retiring.push_back(r);
            }
            s->work_cv.notify_all();
        }
        if (!work) {
            if (s->active.empty())
                s->cv.wait(lk, [&] {
                    return !s->ready.empty() || (s->stop && s->queue.empty() && s->inflight == 0);
                });
            else
                s->cv.wait_for(lk, std::chrono::microseconds(30));
        }
    }
}

}  // namespace

extern "C" {

int fi_serve_create(int max_inflight, double reserve_gb, fi_server** out)
{
    if (!out || max_inflight < 1 || !(reserve_gb >= 0.0)) return FI_E_ARG;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FI_E_CUDA;
    fi_server* s = new fi_server();
    s->device = dev;
    s->max_inflight = max_inflight;
    s->reserve = (size_t)fmin(reserve_gb * 1e9, 1.8e19);
    {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) s->device_total = tot;
    }
    s->t0 = std::chrono::steady_clock::now();
    s->th = std::thread(run, s);
    for (int i = 0; i < kWorkers; ++i) s->workers.emplace_back(worker, s);
    *out = s;
    return FI_OK;
}

int fi_serve_submit(fi_server* s, const fi_request* q, uint64_t* id)
{
    if (!s || !q || !id || !q->z_bed || !q->H_ice || !(q->dtt > 0.0) || !(q->t_end >= q->t0)) return FI_E_ARG;
    Req* r = new Req();
    r->p = q->p;
    r->nxi = q->nx_ice;
    r->nyi = q->ny_ice;
    r->dx = q->dx;
    r->dy = q->dy;
    if (int rc = fi_padded_dims(&q->p, q->nx_ice, q->ny_ice, q->dx, q->dy, r->pd)) {
        delete r;
        return rc;
    }
    const size_t ni = (size_t)q->nx_ice * q->ny_ice, np = (size_t)r->pd[0] * r->pd[1];
    r->z_bed.assign(q->z_bed, q->z_bed + ni);
    r->H.assign(q->H_ice, q->H_ice + ni);
    if (q->H_ref) r->Href.assign(q->H_ref, q->H_ref + ni);
    else r->Href.assign(ni, 0.0);
    if (q->D_lith) r->D.assign(q->D_lith, q->D_lith + np);
    if (q->eta_eff) r->eta.assign(q->eta_eff, q->eta_eff + np);
    if (q->R) r->R.assign(q->R, q->R + np);
    if (q->maskactive) r->mask.assign(q->maskactive, q->maskactive + np);
    r->t0 = q->t0;
    r->t_end = q->t_end;
    r->dtt = q->dtt;
    r->bsl = q->bsl;
    long long ns = 0;
    while (q->t0 + (double)ns * q->dtt < q->t_end) ++ns;
    r->nsteps = ns;
    r->mem_key = np * 2 + (size_t)(q->p.precision & 1);
    memset(&r->info, 0, sizeof(r->info));
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        r->info.t_submit = s->now();
        s->all[r->id] = r;
        s->queue.push_back(r);
        *id = r->id;
    }
    s->work_cv.notify_one();
    return FI_OK;
}

int fi_serve_info(fi_server* s, uint64_t id, fi_request_info* info)
{
    if (!s || !info) return FI_E_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return FI_E_ARG;
    *info = it->second->info;
    return FI_OK;
}

int fi_serve_wait(fi_server* s, uint64_t id, double timeout_s, fi_request_info* info)
{
    if (!s) return FI_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return FI_E_ARG;
    Req* r = it->second;
    const bool ok = s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return r->info.state >= 2; });
    if (info) *info = r->info;
    return ok ? FI_OK : FI_E_TIMEOUT;
}

int fi_serve_result(fi_server* s, uint64_t id, double* w_ice, double* z_bed_ice)
{
    if (!s) return FI_E_ARG;
    Req* r = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(id);
        if (it == s->all.end()) return FI_E_ARG;
        r = it->second;
        if (r->info.state < 2) return FI_E_STATE;
        s->all.erase(it);
    }
    int rc = r->info.state == 2 ? FI_OK : (r->info.status ? r->info.status : FI_E_CUDA);   // 4: FI_E_CANCELLED
    if (rc == FI_OK) {
        if (w_ice) memcpy(w_ice, r->w_out.data(), r->w_out.size() * sizeof(double));
        if (z_bed_ice) memcpy(z_bed_ice, r->zb_out.data(), r->zb_out.size() * sizeof(double));
    }
    delete r;
    return rc;
}

int fi_serve_cancel(fi_server* s, uint64_t id)
{
    if (!s) return FI_E_ARG;
    Req* queued = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(id);
        if (it == s->all.end()) return FI_E_ARG;
        Req* r = it->second;
        if (r->info.state >= 2) return FI_E_STATE;
        for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
            if (*q == r) {
                s->queue.erase(q);
                queued = r;
                break;
            }
        // admitted: the scheduler stops issuing its updates and retires it
        // once the ones in flight have finished
        r->cancel.store(true);
    }
    if (queued) finish(s, queued, 4, FI_E_CANCELLED);
    s->cv.notify_all();
    s->work_cv.notify_all();
    return FI_OK;
}

double fi_serve_clock(fi_server* s) { return s ? s->now() : 0.0; }

int fi_batch_update(fi_handle* const* hs, int n, double time, fi_bsl* bsl)
{
    if (!hs || n < 0 || !bsl) return FI_E_ARG;
    for (int i = 0; i < n; ++i) {
        if (!hs[i]) return FI_E_ARG;
        if (int rc = fi_update_async(hs[i], nullptr, time, &bsl[i])) return rc;
    }
    return FI_OK;
}

int fi_batch_synchronize(fi_handle* const* hs, int n, int32_t* status)
{
    if (!hs || n < 0) return FI_E_ARG;
    int first = FI_OK;
    for (int i = 0; i < n; ++i) {
        const int rc = hs[i] ? fi_synchronize(hs[i]) : FI_E_ARG;
        if (status) status[i] = rc;
        if (rc && first == FI_OK) first = rc;
    }
    return first;
}

int fi_serve_destroy(fi_server* s)
{
    if (!s) return FI_E_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    s->work_cv.notify_all();
    if (s->th.joinable()) s->th.join();
    for (auto& w : s->workers)
        if (w.joinable()) w.join();
    for (auto& kv : s->all) delete kv.second;
    delete s;
    return FI_OK;
}

}  // extern "C"
