// Serving front end: a queue of slice requests run by a pool of contexts on
// one GPU under a device-memory budget.
//
// The reference runs one simulation per process (main.cpp: LoadParameters ->
// Simulate -> save) and has no server; the serving layer is new.  Each worker
// thread owns one bs_ctx (one CUDA stream), so admitted requests run
// concurrently on the GPU.  Admission: a request goes to an idle worker when
// the device bytes of all contexts, with that worker grown to the request's
// estimate (bs_estimate_bytes), stay within the budget.  Among the queued
// requests that fit, the cheapest (pixels x spheres x directions) starts
// first; a request passed by later ones 8 times starts next in any case.
// Each context's stream gets a priority by the cost of its request, so that
// the blocks of short requests are scheduled ahead of those of a long slice
// already running, and with two or more workers the last third of them are
// fast lanes that only take short requests.  When the oldest request fits
// nowhere, idle workers give their buffers back.  Contexts keep their tables
// between requests (bs_set_lut_reuse) and a request goes preferably to the
// worker that last ran the same scene.  Every kernel is deterministic, so a
// result does not depend on what else runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bimsim_gb300.h"

namespace bs {
void set_last_error(const char* msg);
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

constexpr int MAX_SKIPS = 8;  // a queued request is passed at most this often
// With two or more workers the last third of them (at least one) only take
// requests of at most this many (pixel, sphere, wave) interactions, so that
// short requests find contexts even while long slices hold all the others.
constexpr double FAST_LANE_COST = 1e11;

bs_status set_error(bs_status st, const std::string& msg) {
    bs::set_last_error(msg.c_str());
    return st;
}

// FNV-1a over the bytes that decide a context's tables: parameters, spheres
// and precision (the directions do not enter the tables).
uint64_t scene_signature(const bs_params& p, const std::vector<bs_sphere>& s, int prec) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* d, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(d);
        for (size_t i = 0; i < n; i++) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    mix(&p, sizeof(p));
    if (!s.empty()) mix(s.data(), s.size() * sizeof(bs_sphere));
    mix(&prec, sizeof(prec));
    return h;
}

struct Request {
    uint64_t id = 0;
    bs_params prm{};
    std::vector<bs_sphere> spheres;
    std::vector<double> waves;  // empty: compat sampler with nk directions
    int32_t nk = 0;
    int32_t prec = 0;
    int32_t image = 0;
    size_t est = 0;            // device bytes at its own table budget
    double cost = 0;           // work estimate for the order and the stream priority
    uint64_t lut_budget = 0;   // table budget the request runs with (0 = all tables at once)
    uint64_t sig = 0;
    uint64_t shape = 0;        // sig, direction count and table budget: equal shapes allocate equal buffers
    int skipped = 0;
    int state = 0;             // 0 queued, 1 running, 2 done
    bs_status status = BS_OK;
    std::string err;
    std::vector<float> out;
    bs_result_info info{};
    Clock::time_point t_submit, t_start, t_done;
};

struct Worker {
    int index = 0;
    std::thread th;
    bs_ctx* ctx = nullptr;
    uint64_t sig = 0;       // scene whose tables the context holds (0: none)
    uint64_t shape = 0;     // shape of the last request the buffers were sized for (0: none)
    size_t bytes = 0;       // device bytes the context holds
    size_t run_bytes = 0;   // bound on the device bytes while the current job runs
    Request* job = nullptr;
    int prio = 0;           // stream priority of the context
};

// Work of a request in (pixel, sphere, wave) interactions, near-field pixels
// for a scene without spheres.
double request_cost(const bs_params& p, size_t ns, int nk) {
    const double R = (double)p.resolution * p.supersample * (2.0 * p.padding + 1.0);
    return R * R * (double)std::max<size_t>(ns, 1) * (double)std::max(nk, 1);
}

// Stream priority tier of a request: 0 (scheduled first) for the cheapest,
// one more per factor of ten of work above 1e10 interactions.
int cost_tier(double cost) {
    int t = 0;
    for (double c = 1e10; cost > c && t < 8; c *= 10) t++;
    return t;
}

}  // namespace

struct bs_server {
    bs_server_config cfg{};
    int device = 0;
    int prio_least = 0, prio_greatest = 0;  // stream priority range of the device
    size_t budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<std::unique_ptr<Worker>> workers;
    uint64_t next_id = 1;
    bool stop = false;
    int64_t submitted = 0, completed = 0, failed = 0, reuses = 0, running = 0;
    std::vector<double> latencies;
    size_t peak = 0;

    // Device bytes of every context, a busy one counted at least at its job's estimate.
    size_t in_use() const {
        size_t t = 0;
        for (const auto& w : workers) t += w->job ? w->run_bytes : w->bytes;
        return t;
    }

    // Bound on the device bytes of w's context while it runs r.  Buffers only
    // grow, each to the larger of its held and needed size, so a request of
    // another shape can leave the context with up to held + estimate bytes; one
    // of the same shape needs no more than the larger of the two.
    static size_t need(const Worker& w, const Request& r) {
        if (w.bytes == 0) return r.est;
        return r.shape == w.shape ? std::max(w.bytes, r.est) : w.bytes + r.est;
    }

    bool fits(const Worker& w, const Request& r) const {
        const size_t u = in_use() - w.bytes + need(w, r);
        return u <= budget;
    }

    // Can worker w start r now (under mu)?
    bool usable(const Worker& w, const Request& r) const {
        if (r.sig != w.sig) {
            for (const auto& v : workers)  // an idle worker already holds this scene's tables
                if (v.get() != &w && !v->job && v->sig == r.sig) return false;
        }
        return fits(w, r);
    }

    // Next request worker w may start (under mu), or nullptr: the cheapest
    // that it can start, so that short requests do not queue behind long
    // ones; a request passed MAX_SKIPS times by later ones is next in any case.
    bool fast_lane(const Worker& w) const {
        const int n = (int)workers.size();
        return n >= 2 && w.index >= n - std::max(1, n / 3);
    }

    Request* pick(Worker& w) {
        const bool fast = fast_lane(w);
        size_t best = queue.size();
        for (size_t i = 0; i < queue.size(); i++) {
            Request* r = queue[i];
            // the head waits no longer (the fast lane, which can never start a long head, goes on)
            if (i > 0 && queue[0]->skipped >= MAX_SKIPS && !(fast && queue[0]->cost > FAST_LANE_COST)) break;
            if (fast && r->cost > FAST_LANE_COST) continue;
            if (!usable(w, *r)) continue;
            if (best == queue.size() || r->cost < queue[best]->cost) best = i;
        }
        if (best == queue.size()) return nullptr;
        for (size_t j = 0; j < best; j++) queue[j]->skipped++;
        Request* r = queue[best];
        queue.erase(queue.begin() + (long)best);
        return r;
    }

    // The head request fits no worker as things stand.
    bool head_blocked() const {
        if (queue.empty()) return false;
        for (const auto& w : workers)
            if (!w->job && fits(*w, *queue[0])) return false;
        return true;
    }

    size_t run(Worker& w, Request& r);
    void loop(Worker& w);
};

// Runs r on w's context without the lock; returns the context's device bytes
// afterwards (w.bytes itself is only written under the lock).
size_t bs_server::run(Worker& w, Request& r) {
    if (cfg.dry_run) {
        std::this_thread::sleep_for(std::chrono::milliseconds(1));
        r.out.assign((size_t)r.prm.resolution * r.prm.resolution, (float)r.id);
        r.status = BS_OK;
        return w.run_bytes;  // what a context could hold afterwards: the admission bound
    }
    bs_ctx* c = w.ctx;
    cudaSetDevice(device);
    bs_status st = BS_OK;
    // cheaper requests on higher-priority streams: their blocks are scheduled
    // ahead of those of a long slice running on another worker
    const int prio = prio_greatest + std::min(cost_tier(r.cost), prio_least - prio_greatest);
    if (prio != w.prio) {
        st = bs_set_stream_priority(c, prio);
        if (st == BS_OK) w.prio = prio;
    }
    if (st == BS_OK) st = bs_set_params(c, &r.prm);
    if (st == BS_OK) st = bs_set_spheres(c, r.spheres.data(), (int32_t)r.spheres.size());
    if (st == BS_OK && !r.prm.plane_wave) {
        st = r.waves.empty() ? bs_sample_waves_compat(c, r.nk)
                             : bs_set_waves(c, r.waves.data(), (int32_t)(r.waves.size() / 3));
    }
    // an explicit table budget, so the plan never depends on what else holds memory
    if (st == BS_OK) st = bs_set_lut_budget(c, r.lut_budget ? (size_t)r.lut_budget : ((size_t)1 << 62));
    if (st == BS_OK) st = bs_simulate(c, (bs_precision)r.prec);
    if (st == BS_OK) {
        r.out.resize((size_t)r.prm.resolution * r.prm.resolution);
        st = bs_get_image(c, (bs_image_kind)r.image, r.out.data(), r.out.size());
    }
    if (st == BS_OK) {
        bs_stats s{};
        bs_get_stats(c, &s);
        r.info.ms_gpu = s.ms_total;
        r.info.lut_reused = (r.prm.lut_us && r.prm.scalar && !r.spheres.empty() && s.lut_tables_built == 0) ? 1 : 0;
    } else {
        r.err = bs_last_error();
    }
    r.status = st;
    bs_info inf{};
    return bs_get_info(c, &inf) == BS_OK ? (size_t)inf.device_bytes : w.bytes;
}

void bs_server::loop(Worker& w) {
    if (!cfg.dry_run) cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        Request* r = nullptr;
        cv_work.wait(lk, [&] {
            if (stop) return true;
            r = pick(w);
            if (r) return true;
            // nothing fits: give the buffers back if that is what blocks the head request
            if (w.bytes > 0 && head_blocked()) {
                if (!cfg.dry_run) bs_release_buffers(w.ctx);
                w.bytes = 0;
                w.sig = 0;
                w.shape = 0;
                r = pick(w);
                cv_work.notify_all();
                return r != nullptr;
            }
            return false;
        });
        if (!r) return;  // stop
        w.run_bytes = need(w, *r);
        w.job = r;
        r->state = 1;
        r->t_start = Clock::now();
        running++;
        peak = std::max(peak, in_use());
        lk.unlock();
        const size_t held = run(w, *r);
        lk.lock();
        w.bytes = held;
        r->t_done = Clock::now();
        r->info.ms_queued = ms_between(r->t_submit, r->t_start);
        r->info.ms_total = ms_between(r->t_submit, r->t_done);
        r->info.status = r->status;
        r->info.worker = w.index;
        w.sig = r->status == BS_OK ? r->sig : 0;
        w.shape = r->status == BS_OK ? r->shape : 0;
        w.job = nullptr;
        r->state = 2;
        running--;
        if (r->status == BS_OK) {
            completed++;
            latencies.push_back(r->info.ms_total);
            reuses += r->info.lut_reused;
        } else {
            failed++;
        }
        peak = std::max(peak, in_use());
        cv_done.notify_all();
        cv_work.notify_all();
        if (stop) return;
    }
}

extern "C" {

bs_status bs_server_create(const bs_server_config* cfg, bs_server** out) {
    if (!cfg || !out) return set_error(BS_ERR_ARG, "bs_server_create: null argument");
    if (cfg->workers < 0 || cfg->workers > 64) return set_error(BS_ERR_ARG, "bs_server_create: workers must be 0..64");
    std::unique_ptr<bs_server> s(new bs_server());
    s->cfg = *cfg;
    const int nw = cfg->workers ? cfg->workers : 4;
    if (cfg->dry_run) {
        if (!cfg->hbm_budget) return set_error(BS_ERR_ARG, "bs_server_create: a dry run needs an explicit budget");
        s->budget = cfg->hbm_budget;
    } else {
        cudaError_t e = cudaGetDevice(&s->device);
        size_t free_b = 0, total_b = 0;
        if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
        if (e != cudaSuccess) return set_error(BS_ERR_CUDA, std::string("bs_server_create: ") + cudaGetErrorString(e));
        s->budget = cfg->hbm_budget ? cfg->hbm_budget : (size_t)(0.80 * (double)free_b);
        if (cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest) != cudaSuccess)
            s->prio_least = s->prio_greatest = 0;
    }
    bs_params p0{};
    p0.lambda = 1;
    p0.amplitude = 1;
    p0.k_dir[2] = 1;
    p0.condenser[1] = 1;
    p0.objective[1] = 1;
    p0.plane_min[0] = p0.plane_min[1] = -1;
    p0.plane_max[0] = p0.plane_max[1] = 1;
    p0.plane_normal[2] = 1;
    p0.resolution = 1;
    p0.supersample = 1;
    p0.scalar = 1;
    for (int i = 0; i < nw; i++) {
        std::unique_ptr<Worker> w(new Worker());
        w->index = i;
        if (!cfg->dry_run) {
            bs_status st = bs_create(&p0, &w->ctx);
            if (st == BS_OK) st = bs_set_lut_reuse(w->ctx, 1);
            if (st != BS_OK) {
                for (auto& v : s->workers) bs_destroy(v->ctx);
                if (w->ctx) bs_destroy(w->ctx);
                return st;  // message already set
            }
        }
        s->workers.push_back(std::move(w));
    }
    bs_server* srv = s.release();
    for (auto& w : srv->workers) {
        Worker* wp = w.get();
        wp->th = std::thread([srv, wp] { srv->loop(*wp); });
    }
    *out = srv;
    return BS_OK;
}

bs_status bs_server_destroy(bs_server* s) {
    if (!s) return BS_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Request* r : s->queue) {
            r->state = 2;
            r->status = BS_ERR_STATE;
            r->err = "server stopped before the request started";
        }
        s->queue.clear();
    }
    s->cv_work.notify_all();
    for (auto& w : s->workers)
        if (w->th.joinable()) w->th.join();
    for (auto& w : s->workers)
        if (w->ctx) bs_destroy(w->ctx);
    delete s;
    return BS_OK;
}

bs_status bs_submit(bs_server* s, const bs_request* q, uint64_t* ticket) {
    if (!s || !q || !ticket) return set_error(BS_ERR_ARG, "bs_submit: null argument");
    if (q->n_spheres < 0 || (q->n_spheres > 0 && !q->spheres))
        return set_error(BS_ERR_ARG, "bs_submit: bad sphere list");
    if (!q->params.plane_wave && q->n_waves < 1) return set_error(BS_ERR_ARG, "bs_submit: need at least one wave");
    if (q->precision != BS_PREC_FP64 && q->precision != BS_PREC_MIXED)
        return set_error(BS_ERR_ARG, "bs_submit: unknown precision");
    if (q->image < BS_IMG_INTENSITY || q->image > BS_IMG_TRANSMITTANCE)
        return set_error(BS_ERR_ARG, "bs_submit: unknown image kind");
    std::unique_ptr<Request> r(new Request());
    r->prm = q->params;
    r->spheres.assign(q->spheres, q->spheres + q->n_spheres);
    r->nk = q->params.plane_wave ? 1 : q->n_waves;
    if (q->waves && !q->params.plane_wave) r->waves.assign(q->waves, q->waves + 3 * (size_t)q->n_waves);
    r->prec = q->precision;
    r->image = q->image;
    // all tables at once if that fits the budget, else the largest table budget that does
    uint64_t est = 0, est_one = 0;
    bs_status st = bs_estimate_bytes(&r->prm, r->spheres.data(), q->n_spheres, r->nk, (bs_precision)r->prec, 0, &est);
    if (st != BS_OK) return st;
    r->lut_budget = 0;
    if (est > s->budget) {
        // the fixed part is what remains with the smallest table budget that holds one sphere at a time
        uint64_t lo = 1, hi = s->budget;
        bool any = false;
        for (int it = 0; it < 48 && lo < hi; it++) {
            uint64_t mid = lo + (hi - lo) / 2;
            if (bs_estimate_bytes(&r->prm, r->spheres.data(), q->n_spheres, r->nk, (bs_precision)r->prec, mid,
                                  &est_one) == BS_OK &&
                est_one <= s->budget) {
                lo = mid + 1;
                any = true;
            } else {
                hi = mid;
            }
        }
        uint64_t cap = lo > 1 ? lo - 1 : 0;
        if (!any || cap == 0 ||
            bs_estimate_bytes(&r->prm, r->spheres.data(), q->n_spheres, r->nk, (bs_precision)r->prec, cap, &est) !=
                BS_OK ||
            est > s->budget) {
            char msg[160];
            snprintf(msg, sizeof msg, "bs_submit: the request needs more than the budget of %llu bytes",
                     (unsigned long long)s->budget);
            return set_error(BS_ERR_NOMEM, msg);
        }
        r->lut_budget = cap;
    }
    r->est = (size_t)est;
    r->cost = request_cost(r->prm, r->spheres.size(), r->nk);
    r->sig = scene_signature(r->prm, r->spheres, r->prec);
    {
        uint64_t h = r->sig;
        for (uint64_t v : {(uint64_t)(uint32_t)r->nk, (uint64_t)r->lut_budget}) h = (h ^ v) * 1099511628211ull;
        r->shape = h;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_error(BS_ERR_STATE, "bs_submit: server is stopping");
    r->id = s->next_id++;
    r->t_submit = Clock::now();
    *ticket = r->id;
    s->queue.push_back(r.get());
    s->reqs[r->id] = std::move(r);
    s->submitted++;
    s->cv_work.notify_all();
    return BS_OK;
}

bs_status bs_poll(bs_server* s, uint64_t ticket, int32_t* done) {
    if (!s || !done) return set_error(BS_ERR_ARG, "bs_poll: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(BS_ERR_ARG, "bs_poll: unknown ticket");
    *done = it->second->state == 2;
    return BS_OK;
}

bs_status bs_wait(bs_server* s, uint64_t ticket, double timeout_s) {
    if (!s) return set_error(BS_ERR_ARG, "bs_wait: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(BS_ERR_ARG, "bs_wait: unknown ticket");
    Request* r = it->second.get();
    auto ready = [r] { return r->state == 2; };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
        return set_error(BS_ERR_TIMEOUT, "bs_wait: request not finished in time");
    }
    return BS_OK;
}

bs_status bs_fetch(bs_server* s, uint64_t ticket, float* host, size_t count, bs_result_info* info) {
    if (!s) return set_error(BS_ERR_ARG, "bs_fetch: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(BS_ERR_ARG, "bs_fetch: unknown ticket");
    Request* r = it->second.get();
    if (r->state != 2) return set_error(BS_ERR_NOTREADY, "bs_fetch: request not finished");
    if (r->status == BS_OK && host && count < r->out.size()) {
        char msg[96];
        snprintf(msg, sizeof msg, "bs_fetch: need room for %zu floats", r->out.size());
        return set_error(BS_ERR_ARG, msg);
    }
    if (info) *info = r->info;
    bs_status st = r->status;
    if (st == BS_OK) {
        if (host) std::memcpy(host, r->out.data(), r->out.size() * sizeof(float));
    } else {
        set_error(st, r->err);
    }
    s->reqs.erase(it);
    return st;
}

bs_status bs_server_get_stats(bs_server* s, bs_server_stats* out) {
    if (!s || !out) return set_error(BS_ERR_ARG, "bs_server_get_stats: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    bs_server_stats t{};
    t.submitted = s->submitted;
    t.completed = s->completed;
    t.failed = s->failed;
    t.queued = (int64_t)s->queue.size();
    t.running = s->running;
    t.lut_reuses = s->reuses;
    std::vector<double> l = s->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto rank = [&l](double q) {  // nearest-rank percentile
            size_t k = (size_t)std::ceil(q * (double)l.size());
            return l[std::min(l.size(), std::max<size_t>(k, 1)) - 1];
        };
        t.p50_ms = rank(0.50);
        t.p99_ms = rank(0.99);
        double sum = 0;
        for (double v : l) sum += v;
        t.mean_ms = sum / (double)l.size();
        t.max_ms = l.back();
    }
    t.bytes_in_use = s->in_use();
    t.bytes_peak = s->peak;
    t.hbm_budget = s->budget;
    *out = t;
    return BS_OK;
}

}  // extern "C"
