// rts_serve.cpp -- continuous-batching request loop for scattering solves.
//
// Requests (a problem with its inputs and a number of source iterations)
// arrive over time.  One host thread drives one device batch:
//   * admission: arrived requests join the batch in arrival order as long as
//     the context's device bytes plus the request's resident footprint stay
//     under the HBM cap; a request larger than the cap is rejected;
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
//   * a request that has run its iterations is read back (S, FP32) and
//     leaves the batch, freeing its memory for waiting requests.
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
};

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

    std::deque<int64_t> waiting;
    std::vector<Active> active;
    std::vector<double> lat;
    int64_t next = 0, done = 0, rejected = 0, steps = 0, peak = ctx->used_bytes, max_active = 0;
    double work = 0.0;  // cell-direction-iterations completed
    double admit_s = 0.0, step_s = 0.0, retire_s = 0.0;
    const int64_t base_bytes = ctx->used_bytes;
    const auto t0 = clock_type::now();

    while (done + rejected < n) {
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
            rc = rts_batch_add(batch, &d, reqs[r].ibar, reqs[r].B, reqs[r].lambda, &id);
            admit_s += seconds_since(t0) - ta;
            if (rc == RTS_ERR_OVER_BUDGET || rc == RTS_ERR_OUT_OF_MEMORY) {
                if (active.empty()) {  // nothing will free memory: reject
                    waiting.pop_front();
                    ++rejected;
                    continue;
                }
                break;
            }
            if (rc != RTS_OK) {
                rts_batch_destroy(batch);
                return rc;
            }
            const int64_t tiles = rts_group_problem_tiles(batch, id);
            active.push_back(Active{r, id, reqs[r].iterations, fp, tiles,
                                    (double)d.N * (double)d.groups * (double)d.M * (double)d.M, 0,
                                    reqs[r].arrival_s + 0.01 * ctx->serve_slack *
                                                            isolated_estimate(tiles, d.M, reqs[r].iterations,
                                                                              ctx->num_sms)});
            waiting.pop_front();
            peak = std::max(peak, ctx->used_bytes);
        }
        max_active = std::max<int64_t>(max_active, (int64_t)active.size());
        if (active.empty()) {
            if (next < n) {
                const double wait = reqs[next].arrival_s - seconds_since(t0);
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
                continue;
            }
            break;  // only rejected requests were left
        }
        // the pieces this launch runs: (request, first tile, tiles)
        std::vector<size_t> order(active.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::vector<int64_t> take(active.size(), 0);
        if (ctx->serve_policy != 0) {
            auto key = [&](size_t i) {
                if (ctx->serve_policy == 1) return active[i].deadline;
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
            for (size_t i = 0; i < active.size(); ++i) take[i] = active[i].tiles - active[i].pos;
        }
        std::vector<int64_t> ids, first, count;
        for (size_t i = 0; i < active.size(); ++i) {
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
        rc = rts_group_step_pieces(batch, 1, ids.data(), first.data(), count.data(), (int)ids.size(),
                                   ctx->streams[RTS_STREAM_SCATTERING_1]);
        if (rc == RTS_OK) rc = rts_batch_sync(batch, step_timeout_us);
        step_s += seconds_since(t0) - ts;
        if (rc != RTS_OK) {
            rts_batch_destroy(batch);
            return rc;
        }
        for (size_t i = 0; i < active.size(); ++i) {
            active[i].pos += take[i];
            if (take[i] > 0 && active[i].pos == active[i].tiles) {  // the step is complete
                active[i].pos = 0;
                active[i].remaining--;
            }
        }
        ++steps;
        // completions
        for (size_t i = 0; i < active.size();) {
            Active& a = active[i];
            if (a.remaining > 0) {
                ++i;
                continue;
            }
            const rts_request& q = reqs[a.req];
            const double tr = seconds_since(t0);
            rc = rts_batch_read(batch, a.id, q.S_out, nullptr);
            if (rc == RTS_OK) rc = rts_batch_remove(batch, a.id);
            retire_s += seconds_since(t0) - tr;
            if (rc != RTS_OK) {
                rts_batch_destroy(batch);
                return rc;
            }
            const double l = (seconds_since(t0) - q.arrival_s) * 1e3;
            if (latency_ms) latency_ms[a.req] = l;
            lat.push_back(l);
            work += (double)q.desc.N * (double)q.desc.groups * (double)q.desc.M * (double)q.iterations;
            ++done;
            active[i] = active.back();
            active.pop_back();
        }
    }
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
