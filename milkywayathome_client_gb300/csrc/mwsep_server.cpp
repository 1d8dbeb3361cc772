/* mwsep_server.cpp -- the serving loop: continuous batching of evaluation
 * requests over the wedges resident in a context.
 *
 * The server owns `lanes` execution lanes.  A lane is a context sharing the
 * parent's resident wedges (no copy of the tables) with its own CUDA stream,
 * engine buffers and captured graph, driven by one dispatcher thread.  A
 * dispatcher that is free takes the queued requests of the oldest request's
 * precision in arrival order (up to max_batch, and -- with target_batch_ms
 * set -- until their predicted device time reaches it) and evaluates them as
 * one engine batch; requests that arrive meanwhile go to the next lane that
 * frees up, so batches on different lanes overlap on the GPU.  The
 * prediction is a request's density points (mwsep_ctx_wedge_points) times
 * the time per point of its precision, which the lanes measure on every
 * batch they run (a moving average, contention from the other lanes
 * included).  A batch that would push the lane past its share of the
 * device-memory budget is split in half until it fits (admission by HBM
 * footprint), and with max_queued set a submit finding that many requests
 * waiting is refused with MWSEP_ERR_BUSY.
 *
 * A request's result is the same whichever lane or batch runs it: the
 * reduction order of an evaluation depends only on its wedge's tile shape.
 *
 * Waits are bounded: mwsep_server_wait gives up after its timeout with
 * MWSEP_ERR_TIMEOUT, and a request cancelled while still queued completes
 * with MWSEP_ERR_CANCELLED.
 */
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "milkyway_separation_gb300.h"
#include "mwsep_status.h"

extern "C" mwsep_ctx* mwsep_ctx_lane(mwsep_ctx* parent);

namespace {

using Clock = std::chrono::steady_clock;

struct Request
{
    uint64_t id;
    int wedge;
    int precision;
    std::vector<double> theta;
    Clock::time_point submitted;
    double points = 0.0; /* density points of one evaluation of its wedge */
    bool done = false;
    bool started = false;
    int status = MWSEP_OK;
    mwsep_result result;
    double latency_s = 0.0;
};

} // namespace

struct mwsep_server
{
    mwsep_ctx* parent = nullptr;
    mwsep_server_config cfg;
    std::vector<mwsep_ctx*> lanes;
    std::vector<std::thread> threads;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, Request*> all;
    uint64_t next_id = 1;
    bool stop = false;

    /* device time per density point of each precision (plain FP64,
     * compensated, double-float), in ns, seeded with GB300's full-size rates
     * (1.72e10 points in 2.06 s, 15.6 ms, 165 ms) and refreshed from every
     * batch */
    double ns_per_point[3] = {0.12, 0.00091, 0.0096};

    /* statistics */
    std::vector<double> latencies;
    long long batches = 0, evaluated = 0, cancelled = 0, failed = 0, refused = 0, max_queue = 0;
    Clock::time_point first_submit, last_done;
    bool any = false;
};

namespace {

void lane_loop(mwsep_server* s, int lane)
{
    mwsep_ctx* ctx = s->lanes[lane];
    std::vector<Request*> batch;
    std::vector<mwsep_request> reqs;
    std::vector<mwsep_result> out;
    for (;;)
    {
        batch.clear();
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_work.wait(lock, [&] { return s->stop || !s->queue.empty(); });
            if (s->stop && s->queue.empty()) return;
            const int precision = s->queue.front()->precision;
            const double cap_ms = s->cfg.target_batch_ms;
            double predicted_ms = 0.0;
            for (auto it = s->queue.begin(); it != s->queue.end() && (int)batch.size() < s->cfg.max_batch;)
            {
                if ((*it)->precision == precision)
                {
                    const double ms = (*it)->points * s->ns_per_point[precision] * 1e-6;
                    if (cap_ms > 0.0 && !batch.empty() && predicted_ms + ms > cap_ms) break;
                    predicted_ms += ms;
                    (*it)->started = true;
                    batch.push_back(*it);
                    it = s->queue.erase(it);
                }
                else
                    ++it;
            }
        }
        /* evaluate; split in halves while the lane's memory share refuses it */
        const auto t_batch = Clock::now();
        double batch_points = 0.0;
        for (const Request* r : batch) batch_points += r->points;
        size_t done = 0;
        while (done < batch.size())
        {
            size_t take = batch.size() - done;
            int rc;
            for (;;)
            {
                reqs.resize(take);
                out.resize(take);
                for (size_t i = 0; i < take; ++i)
                {
                    reqs[i].wedge = batch[done + i]->wedge;
                    reqs[i].theta = batch[done + i]->theta.data();
                }
                rc = mwsep_ctx_evaluate_requests(ctx, (int)take, reqs.data(), batch[done]->precision, out.data());
                if (rc == MWSEP_ERR_BUDGET && take > 1)
                {
                    take = (take + 1) / 2;
                    continue;
                }
                break;
            }
            const auto now = Clock::now();
            std::lock_guard<std::mutex> lock(s->mu);
            for (size_t i = 0; i < take; ++i)
            {
                Request* r = batch[done + i];
                r->status = rc;
                if (rc == MWSEP_OK) r->result = out[i];
                r->latency_s = std::chrono::duration<double>(now - r->submitted).count();
                r->done = true;
                if (rc == MWSEP_OK)
                {
                    s->latencies.push_back(r->latency_s);
                    ++s->evaluated;
                }
                else
                    ++s->failed;
            }
            ++s->batches;
            s->last_done = now;
            if (done + take == batch.size() && rc == MWSEP_OK && batch_points > 0.0)
            {
                const int p = batch.front()->precision;
                const double ns = std::chrono::duration<double>(now - t_batch).count() * 1e9 / batch_points;
                s->ns_per_point[p] = 0.7 * s->ns_per_point[p] + 0.3 * ns;
            }
            s->cv_done.notify_all();
            done += take;
        }
    }
}

double percentile(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

} // namespace

extern "C" int mwsep_server_create(mwsep_ctx* ctx, const mwsep_server_config* cfg, mwsep_server** out)
{
    if (!ctx || !out) return mwsep_fail(MWSEP_ERR_ARG);
    *out = nullptr;
    mwsep_server* s = new (std::nothrow) mwsep_server();
    if (!s) return mwsep_fail(MWSEP_ERR_NOMEM);
    s->parent = ctx;
    s->cfg.lanes = 2;
    s->cfg.max_batch = 256;
    s->cfg.lane_hbm_bytes = 0;
    s->cfg.target_batch_ms = 0.0;
    s->cfg.max_queued = 0;
    if (cfg) s->cfg = *cfg;
    if (s->cfg.lanes < 1 || s->cfg.lanes > 16 || s->cfg.max_batch < 1 || !(s->cfg.target_batch_ms >= 0.0) ||
        s->cfg.max_queued < 0)
    {
        delete s;
        return mwsep_fail(MWSEP_ERR_ARG);
    }
    for (int i = 0; i < s->cfg.lanes; ++i)
    {
        mwsep_ctx* lane = mwsep_ctx_lane(ctx);
        if (!lane)
        {
            for (mwsep_ctx* l : s->lanes) mwsep_ctx_destroy(l);
            delete s;
            return mwsep_fail(MWSEP_ERR_CUDA);
        }
        if (s->cfg.lane_hbm_bytes) mwsep_ctx_set_hbm_budget(lane, s->cfg.lane_hbm_bytes);
        s->lanes.push_back(lane);
    }
    for (int i = 0; i < s->cfg.lanes; ++i) s->threads.emplace_back(lane_loop, s, i);
    *out = s;
    return MWSEP_OK;
}

extern "C" int mwsep_server_submit(mwsep_server* s, int wedge, const double* theta, int precision,
                                   unsigned long long* id)
{
    if (!s || !theta || !id) return mwsep_fail(MWSEP_ERR_ARG);
    if (precision != MWSEP_PLAIN_F64 && precision != MWSEP_MIXED_F32 && precision != MWSEP_PLAIN_DF)
        return mwsep_fail(MWSEP_ERR_ARG);
    const int n = mwsep_ctx_wedge_theta_count(s->parent, wedge);
    if (n < 0) return mwsep_fail(MWSEP_ERR_ARG);
    double points = 0.0;
    if (mwsep_ctx_wedge_points(s->parent, wedge, &points) != MWSEP_OK) return mwsep_fail(MWSEP_ERR_ARG);
    Request* r = new (std::nothrow) Request();
    if (!r) return mwsep_fail(MWSEP_ERR_NOMEM);
    r->wedge = wedge;
    r->points = points;
    r->precision = precision;
    r->theta.assign(theta, theta + n);
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->stop)
        {
            delete r;
            return mwsep_fail(MWSEP_ERR_STATE);
        }
        if (s->cfg.max_queued > 0 && (long long)s->queue.size() >= s->cfg.max_queued)
        {
            ++s->refused;
            delete r;
            return mwsep_fail(MWSEP_ERR_BUSY);
        }
        r->id = s->next_id++;
        if (!s->any)
        {
            s->first_submit = r->submitted;
            s->any = true;
        }
        s->queue.push_back(r);
        s->max_queue = std::max(s->max_queue, (long long)s->queue.size());
        s->all[r->id] = r;
        *id = r->id;
    }
    s->cv_work.notify_one();
    return MWSEP_OK;
}

extern "C" int mwsep_server_cancel(mwsep_server* s, unsigned long long id)
{
    if (!s) return mwsep_fail(MWSEP_ERR_ARG);
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return mwsep_fail(MWSEP_ERR_ARG);
    Request* r = it->second;
    if (r->started || r->done) return mwsep_fail(MWSEP_ERR_STATE);
    s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), r), s->queue.end());
    r->done = true;
    r->status = MWSEP_ERR_CANCELLED;
    ++s->cancelled;
    s->cv_done.notify_all();
    return MWSEP_OK;
}

extern "C" int mwsep_server_wait(mwsep_server* s, unsigned long long id, double timeout_s, mwsep_result* out)
{
    if (!s) return mwsep_fail(MWSEP_ERR_ARG);
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return mwsep_fail(MWSEP_ERR_ARG);
    Request* r = it->second;
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(std::max(timeout_s, 0.0)));
    if (!s->cv_done.wait_until(lock, deadline, [&] { return r->done; })) return mwsep_fail(MWSEP_ERR_TIMEOUT);
    const int status = r->status;
    if (out && status == MWSEP_OK) *out = r->result;
    s->all.erase(it);
    delete r;
    return status == MWSEP_OK ? MWSEP_OK : mwsep_fail(status);
}

extern "C" int mwsep_server_get_stats(mwsep_server* s, mwsep_server_stats* out)
{
    if (!s || !out) return mwsep_fail(MWSEP_ERR_ARG);
    std::lock_guard<std::mutex> lock(s->mu);
    memset(out, 0, sizeof(*out));
    out->completed = s->evaluated;
    out->failed = s->failed;
    out->cancelled = s->cancelled;
    out->batches = s->batches;
    out->queued = (long long)s->queue.size();
    out->mean_batch = s->batches ? (double)(s->evaluated + s->failed) / (double)s->batches : 0.0;
    out->p50_latency_s = percentile(s->latencies, 0.50);
    out->p99_latency_s = percentile(s->latencies, 0.99);
    out->max_latency_s = s->latencies.empty() ? 0.0 : *std::max_element(s->latencies.begin(), s->latencies.end());
    const double span = s->any ? std::chrono::duration<double>(s->last_done - s->first_submit).count() : 0.0;
    out->evals_per_s = span > 0 ? (double)s->evaluated / span : 0.0;
    out->refused = s->refused;
    out->max_queue = s->max_queue;
    return MWSEP_OK;
}

extern "C" int mwsep_server_reset_stats(mwsep_server* s)
{
    if (!s) return mwsep_fail(MWSEP_ERR_ARG);
    std::lock_guard<std::mutex> lock(s->mu);
    s->latencies.clear();
    s->batches = s->evaluated = s->cancelled = s->failed = s->refused = 0;
    s->max_queue = (long long)s->queue.size();
    s->any = false;
    return MWSEP_OK;
}

extern "C" int mwsep_server_destroy(mwsep_server* s)
{
    if (!s) return mwsep_fail(MWSEP_ERR_ARG);
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        /* queued requests are cancelled; running batches finish */
        for (Request* r : s->queue)
        {
            r->done = true;
            r->status = MWSEP_ERR_CANCELLED;
        }
        s->queue.clear();
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    for (std::thread& t : s->threads) t.join();
    for (mwsep_ctx* l : s->lanes) mwsep_ctx_destroy(l);
    for (auto& kv : s->all) delete kv.second;
    delete s;
    return MWSEP_OK;
}
