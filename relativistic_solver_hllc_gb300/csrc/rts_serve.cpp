// rts_serve.cpp -- continuous-batching request loop for scattering solves.
//
// Requests (a problem with its inputs and a number of source iterations)
// arrive over time.  One host thread drives one device batch:
//   * admission: arrived requests join the batch in arrival order as long as
//     the context's device bytes plus the request's resident footprint stay
//     under the HBM cap; a request larger than the cap is rejected.  Its
//     set-up (W, copies, split) is queued on a low-priority stream of its own
//     and overlaps the running steps; the request takes part in steps once
//     that set-up has finished;
//   * every step advances resident requests by one source iteration in one
//     grouped tcgen05 launch, so requests that arrive while others run share
//     the device from their first step on.  Which ones (RTS_TUNE_SERVE_POLICY):
//     earliest deadline first (deadline = arrival + slack (default 5) x the
//     request's estimated solve time alone: iterations x (launch overhead +
//     its tiles' waves on the SMs)), or least remaining work first (priority = remaining
//     work / (1 + steps waited)), each filling a tile budget per launch that
//     keeps launches short -- a request's step is cut into pieces of tiles
//     when it does not fit, so a large step never holds back an urgent small
//     request for long; or all of them, one whole step each;
//   * a request that has run its iterations is read back (S, FP32) on a copy
//     stream and leaves the batch, freeing its memory for waiting requests.
// The host keeps up to G_INFLIGHT steps queued ahead of the device (each with
// an event), so set-up, retirement and scheduling overlap the running step;
// problem buffers come from a stream-ordered pool, so admitting or retiring a
// request never synchronises the device.
// Latency = completion time - arrival time (host wall clock).  Waits on the
// device are bounded; nothing here blocks forever.
//
// No counterpart in the reference (one solve per process).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "rts_group.h"
#include "rts_internal.h"

namespace {

using clock_type = std::chrono::steady_clock;

double seconds_since(clock_type::time_point t0)
{
    return std::chrono::duration<double>(clock_type::now() - t0).count();
}

double percentile(std::vector<double> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (double)(v.size() - 1);
    const size_t lo = (size_t)std::floor(pos), hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
}

constexpr int G_INFLIGHT = 2;  // steps queued ahead of the device

struct Active {
    int64_t req = 0;
    int64_t id = 0;
    int remaining = 0;
    int64_t bytes = 0;
    int64_t tiles = 0;    // tiles of one step
    double step_work = 0;  // cells x directions^2 of one step
    int waited = 0;       // consecutive steps left out
    double deadline = 0;  // arrival + 2 x estimated isolated solve time (s)
    int64_t pos = 0;      // next tile of the current step (a step may span launches)
    int state = 0;        // -1 set-up queued, 0 running, 1 last step queued, 2 read-back queued
    cudaEvent_t ready = nullptr;   // set-up done (state -1)
    cudaEvent_t copied = nullptr;  // read-back done (state 2)
};

struct Queued {  // a launched step: its completion event and the requests it finishes
    cudaEvent_t done = nullptr;
    std::vector<int64_t> finishing;  // batch ids
};

// Polls an event until it completes or `timeout_us` passes (< 0: no limit).
int wait_event(rts_ctx* ctx, cudaEvent_t ev, int64_t timeout_us)
{
    const auto t0 = clock_type::now();
    for (;;) {
        const cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return RTS_OK;
        if (e != cudaErrorNotReady) return rts_fail(ctx, RTS_ERR_CUDA, "serving: %s", cudaGetErrorString(e));
        if (timeout_us >= 0 && seconds_since(t0) * 1e6 > (double)timeout_us)
            return rts_fail(ctx, RTS_ERR_TIMEOUT, "serving: a step did not finish within %lld us",
                            (long long)timeout_us);
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

// Solve time of a request alone: per step a fixed launch and host overhead
// plus its tiles in waves over the SMs, each tile taking about 1 us per
// 32-direction K-slice (two issuers, measured on GB300 at N = 256 columns).
double isolated_estimate(int64_t tiles, int64_t M, int iterations, int num_sms)
{
    const double waves = std::ceil((double)tiles / (double)num_sms);
    const double tile_s = 1.0e-6 * (double)((M + 31) / 32);
    return (double)iterations * (30e-6 + waves * tile_s);
}

}  // namespace

extern "C" int rts_serve_run(rts_ctx* ctx, const rts_request* reqs, int64_t n, int64_t hbm_cap, int64_t step_timeout_us,
                             double* latency_ms, rts_serve_stats* stats)
{
    if (!ctx || (n > 0 && !reqs) || n < 0 || !stats) return RTS_ERR_INVALID_ARGUMENT;
    for (int64_t i = 0; i < n; ++i) {
        RTS_REQUIRE(ctx, reqs[i].iterations > 0, RTS_ERR_INVALID_ARGUMENT, "request %lld has no iterations",
                    (long long)i);
        RTS_REQUIRE(ctx, i == 0 || reqs[i].arrival_s >= reqs[i - 1].arrival_s, RTS_ERR_INVALID_ARGUMENT,
                    "requests must be sorted by arrival time");
    }
    memset(stats, 0, sizeof(*stats));
    for (int64_t i = 0; i < n; ++i)
        if (latency_ms) latency_ms[i] = -1.0;
    rts_batch* batch = nullptr;
    int rc = rts_batch_create(ctx, &batch);
    if (rc != RTS_OK) return rc;
    if (!ctx->serve_copy && cudaStreamCreateWithFlags(&ctx->serve_copy, cudaStreamNonBlocking) != cudaSuccess) {
        rts_batch_destroy(batch);
        return rts_fail(ctx, RTS_ERR_CUDA, "serving: cannot create the copy stream");
    }
    if (!ctx->serve_admit) {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (cudaStreamCreateWithPriority(&ctx->serve_admit, cudaStreamNonBlocking, least) != cudaSuccess) {
            rts_batch_destroy(batch);
            return rts_fail(ctx, RTS_ERR_CUDA, "serving: cannot create the set-up stream");
        }
    }
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    std::vector<cudaEvent_t> events;  // free list
    auto take_event = [&](cudaEvent_t* ev) {
        if (!events.empty()) {
            *ev = events.back();
            events.pop_back();
            return cudaSuccess;
        }
        return cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    };

    std::deque<int64_t> waiting;
    std::vector<Active> active;
    std::deque<Queued> queued;
    std::vector<double> lat;
    int64_t next = 0, done = 0, rejected = 0, steps = 0, peak = ctx->used_bytes, max_active = 0;
    double work = 0.0;  // cell-direction-iterations completed
    double admit_s = 0.0, step_s = 0.0, retire_s = 0.0;
    const int64_t base_bytes = ctx->used_bytes;
    const auto t0 = clock_type::now();

    auto fail = [&](int code) {
        cudaStreamSynchronize(st);
        cudaStreamSynchronize(ctx->serve_copy);
        for (Queued& q : queued) events.push_back(q.done);
        cudaStreamSynchronize(ctx->serve_admit);
        for (Active& a : active) {
            if (a.copied) events.push_back(a.copied);
            if (a.ready) events.push_back(a.ready);
        }
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        rts_batch_destroy(batch);
        return code;
    };
    // the oldest queued step finished: queue the read-back of every request it completed
    auto finish_step = [&]() -> int {
        Queued& q = queued.front();
        for (int64_t id : q.finishing) {
            for (Active& a : active) {
                if (a.id != id) continue;
                const rts_request& rq = reqs[a.req];
                GProb* p = rts_group_find(batch, id, nullptr);
                if (rq.S_out && p && p->S32 &&
                    cudaMemcpyAsync(rq.S_out, p->S32, (size_t)(p->rows * p->Mout) * 4, cudaMemcpyDeviceToHost,
                                    ctx->serve_copy) != cudaSuccess)
                    return rts_fail(ctx, RTS_ERR_CUDA, "serving: read-back failed");
                if (take_event(&a.copied) != cudaSuccess || cudaEventRecord(a.copied, ctx->serve_copy) != cudaSuccess)
                    return rts_fail(ctx, RTS_ERR_CUDA, "serving: event record failed");
                a.state = 2;
            }
        }
        events.push_back(q.done);
        queued.pop_front();
        return RTS_OK;
    };
    // requests whose read-back has landed leave the batch
    auto retire = [&]() -> int {
        for (size_t i = 0; i < active.size();) {
            Active& a = active[i];
            if (a.state != 2 || cudaEventQuery(a.copied) != cudaSuccess) {
                ++i;
                continue;
            }
            const double tr = seconds_since(t0);
            const rts_request& q = reqs[a.req];
            const int r2 = rts_group_remove_on(batch, a.id, ctx->serve_copy);  // freed after the read-back
            retire_s += seconds_since(t0) - tr;
            if (r2 != RTS_OK) return r2;
            const double l = (seconds_since(t0) - q.arrival_s) * 1e3;
            if (latency_ms) latency_ms[a.req] = l;
            lat.push_back(l);
            work += (double)q.desc.N * (double)q.desc.groups * (double)q.desc.M * (double)q.iterations;
            ++done;
            events.push_back(a.copied);
            active[i] = active.back();
            active.pop_back();
        }
        return RTS_OK;
    };

    while (done + rejected < n) {
        // completed steps and read-backs first: they free memory and slots
        while (!queued.empty() && cudaEventQuery(queued.front().done) == cudaSuccess)
            if ((rc = finish_step()) != RTS_OK) return fail(rc);
        if ((rc = retire()) != RTS_OK) return fail(rc);
        for (Active& a : active)
            if (a.state == -1 && cudaEventQuery(a.ready) == cudaSuccess) {
                a.state = 0;
                events.push_back(a.ready);
                a.ready = nullptr;
            }

        const double now = seconds_since(t0);
        while (next < n && reqs[next].arrival_s <= now) waiting.push_back(next++);
        // admission in arrival order while the HBM cap allows
        while (!waiting.empty()) {
            const int64_t r = waiting.front();
            int64_t fp = 0;
            rts_problem_footprint(&reqs[r].desc, &fp);
            const rts_problem_desc& d = reqs[r].desc;
            // transient set-up scratch: FP64 W and FP32 Ibar staging
            const int64_t scratch = d.M * d.M * 8 + d.N * d.groups * d.M * 4;
            if (base_bytes + fp + scratch > hbm_cap) {  // can never fit
                waiting.pop_front();
                ++rejected;
                continue;
            }
            if (ctx->used_bytes + fp + scratch > hbm_cap && !active.empty()) break;
            int64_t id = 0;
            const double ta = seconds_since(t0);
            rc = rts_batch_add_on(batch, &d, reqs[r].ibar, reqs[r].B, reqs[r].lambda, ctx->serve_admit, false, &id);
            cudaEvent_t ready = nullptr;
            if (rc == RTS_OK && (take_event(&ready) != cudaSuccess || cudaEventRecord(ready, ctx->serve_admit) != cudaSuccess))
                rc = rts_fail(ctx, RTS_ERR_CUDA, "serving: event record failed");
            admit_s += seconds_since(t0) - ta;
            if (rc == RTS_ERR_OVER_BUDGET || rc == RTS_ERR_OUT_OF_MEMORY) {
                if (active.empty()) {  // nothing will free memory: reject
                    waiting.pop_front();
                    ++rejected;
                    continue;
                }
                break;
            }
            if (rc != RTS_OK) return fail(rc);
            const int64_t tiles = rts_group_problem_tiles(batch, id);
            Active a;
            a.req = r;
            a.id = id;
            a.remaining = reqs[r].iterations;
            a.bytes = fp;
            a.tiles = tiles;
            a.step_work = (double)d.N * (double)d.groups * (double)d.M * (double)d.M;
            a.deadline = reqs[r].arrival_s +
                         0.01 * ctx->serve_slack * isolated_estimate(tiles, d.M, reqs[r].iterations, ctx->num_sms);
            a.state = -1;
            a.ready = ready;
            active.push_back(a);
            waiting.pop_front();
            peak = std::max(peak, ctx->used_bytes);
        }
        max_active = std::max<int64_t>(max_active, (int64_t)active.size());

        // requests with iterations still to launch
        std::vector<size_t> order;
        for (size_t i = 0; i < active.size(); ++i)
            if (active[i].state == 0) order.push_back(i);
        if (order.empty() || (int)queued.size() >= G_INFLIGHT) {
            // nothing to launch now: wait for the device (a step or a read-back)
            if (!queued.empty()) {
                const double tw = seconds_since(t0);
                rc = wait_event(ctx, queued.front().done, step_timeout_us);
                step_s += seconds_since(t0) - tw;
                if (rc != RTS_OK) return fail(rc);
                continue;
            }
            bool copying = false;
            for (const Active& a : active) copying |= a.state == 2 || a.state == -1;
            if (copying) {
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                continue;
            }
            if (next < n) {
                const double wait = reqs[next].arrival_s - seconds_since(t0);
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
                continue;
            }
            if (active.empty()) break;  // only rejected requests were left
            continue;
        }
        // the pieces this launch runs: (request, first tile, tiles)
        std::vector<int64_t> take(active.size(), 0);
        if (ctx->serve_policy != 0) {
            auto key = [&](size_t i) {
                if (ctx->serve_policy == 1) return active[i].deadline;
                if (ctx->serve_policy == 3) return reqs[active[i].req].arrival_s;
                return active[i].step_work * active[i].remaining / (1.0 + active[i].waited);
            };
            std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return key(x) < key(y); });
            const int64_t budget = ctx->serve_budget > 0 ? ctx->serve_budget : 8 * (int64_t)ctx->num_sms;
            int64_t left = budget;
            for (size_t i : order) {
                if (left <= 0) break;
                take[i] = std::min(active[i].tiles - active[i].pos, left);
                left -= take[i];
            }
        } else {
            for (size_t i : order) take[i] = active[i].tiles - active[i].pos;
        }
        std::vector<int64_t> ids, first, count;
        for (size_t i : order) {
            if (take[i] > 0) {
                ids.push_back(active[i].id);
                first.push_back(active[i].pos);
                count.push_back(take[i]);
                active[i].waited = 0;
            } else {
                active[i].waited++;
            }
        }
        const double ts = seconds_since(t0);
        rc = rts_group_step_pieces(batch, 1, ids.data(), first.data(), count.data(), (int)ids.size(), st);
        Queued q;
        if (rc == RTS_OK && (take_event(&q.done) != cudaSuccess || cudaEventRecord(q.done, st) != cudaSuccess))
            rc = rts_fail(ctx, RTS_ERR_CUDA, "serving: event record failed");
        step_s += seconds_since(t0) - ts;
        if (rc != RTS_OK) return fail(rc);
        for (size_t i : order) {
            Active& a = active[i];
            a.pos += take[i];
            if (take[i] > 0 && a.pos == a.tiles) {  // the step is complete
                a.pos = 0;
                if (--a.remaining == 0) {
                    a.state = 1;
                    q.finishing.push_back(a.id);
                }
            }
        }
        queued.push_back(q);
        ++steps;
    }
    // a bounded wait reported on the device invalidates the results
    int flag = 0;
    if (cudaStreamSynchronize(ctx->serve_copy) != cudaSuccess || cudaStreamSynchronize(ctx->serve_admit) != cudaSuccess ||
        cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(rts_fail(ctx, RTS_ERR_CUDA, "serving: final synchronisation failed"));
    if (flag) return fail(rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "serving: the batched kernel reported device flag %d", flag));
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    events.clear();
    const double makespan = seconds_since(t0);
    rts_batch_destroy(batch);
    stats->completed = done;
    stats->rejected = rejected;
    stats->max_active = max_active;
    stats->steps = steps;
    stats->makespan_s = makespan;
    stats->throughput = makespan > 0 ? work / makespan : 0.0;
    stats->p50_ms = percentile(lat, 0.50);
    stats->p99_ms = percentile(lat, 0.99);
    double sum = 0, mx = 0;
    for (double v : lat) {
        sum += v;
        mx = std::max(mx, v);
    }
    stats->mean_ms = lat.empty() ? 0.0 : sum / (double)lat.size();
    stats->max_ms = mx;
    stats->peak_bytes = peak;
    stats->admit_s = admit_s;
    stats->step_s = step_s;
    stats->retire_s = retire_s;
    return RTS_OK;
}

extern "C" int rts_host_alloc(int64_t bytes, void** ptr)
{
    if (!ptr || bytes <= 0) return RTS_ERR_INVALID_ARGUMENT;
    *ptr = nullptr;
    if (cudaMallocHost(ptr, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return RTS_ERR_OUT_OF_MEMORY;
    }
    return RTS_OK;
}

extern "C" int rts_host_free(void* ptr)
{
    if (ptr) cudaFreeHost(ptr);
    return RTS_OK;
}
