// Autotuner for the FAST kernels: picks the tile preset, pairs per pipeline stage,
// pipeline depth and pair splits of a plan or a batch by timing candidates on the
// caller's device buffers, and remembers the choice per workload shape.
//
// Search (staged, so a 256^3 capture tunes in seconds):
//   1. every tile preset the kernel family runs, at its own chunk and depth;
//   2. chunk {16, 32, 64} x depth {2, 3, 4} on the two fastest presets;
//   3. pair splits {1, 2, 4} on the winner (plans only; 0 = the plan's own choice).
// Each candidate runs once untimed, then enough timed repetitions (CUDA events on the
// caller's stream) to cover about 20 ms.  The winner is re-run with bin-window checking
// and rejected, in favour of the next fastest, if any bin fell outside its window.
//
// Cache: key = device name + SM count + row type + accumulation + workload shape
// (pairs, T, voxels, deltaT for plans; the ordered list of capture shapes for batches).
// bpgb_tune_cache_save / _load write and read one text line per entry:
//   <key> <tile> <chunk> <stages> <pair_splits> <best_ms>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "bpgb_internal.h"

namespace bpgb {
namespace {

struct TuneEntry {
    int tile = -1, chunk = 0, stages = 0, splits = 0;
    float ms = 0.0f;
};

std::mutex g_mu;
std::map<std::string, TuneEntry> g_cache;

std::string device_tag() {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p{};
    cudaGetDeviceProperties(&p, dev);
    std::string name = p.name;
    for (char &c : name)
        if (c == ' ') c = '_';
    return name + "/sm" + std::to_string(p.multiProcessorCount);
}

struct Candidate {
    int tile, chunk, stages, splits;
    float ms;
};

// Times `run` (which launches one execute on `s`); returns ms per execute, or < 0 when
// the candidate cannot run.
template <typename Run>
float time_candidate(Run &&run, cudaStream_t s) {
    if (run()) return -1.0f;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return -1.0f;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return -1.0f;
    }
    float ms = -1.0f;
    // one timed run sizes the repetitions
    cudaEventRecord(e0, s);
    bool ok = run() == 0;
    cudaEventRecord(e1, s);
    if (ok && cudaEventSynchronize(e1) == cudaSuccess) {
        float one = 0.0f;
        cudaEventElapsedTime(&one, e0, e1);
        const int reps = std::max(1, std::min(10, (int)(20.0f / std::max(one, 1e-3f))));
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps && ok; r++) ok = run() == 0;
        cudaEventRecord(e1, s);
        if (ok && cudaEventSynchronize(e1) == cudaSuccess) {
            float tot = 0.0f;
            cudaEventElapsedTime(&tot, e0, e1);
            ms = tot / reps;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

// The staged search over `make_and_time(tile, chunk, stages, splits)`; `validate`
// re-runs a candidate checked and returns true when every bin stayed in its window.
template <typename MakeTime, typename Validate>
int search(const std::vector<int> &tiles, bool try_splits, MakeTime &&make_and_time,
           Validate &&validate, TuneEntry *best, bpgb_tune_report *rep) {
    std::vector<Candidate> all;
    auto trial = [&](int tile, int chunk, int stages, int splits) {
        for (const Candidate &c : all)
            if (c.tile == tile && c.chunk == chunk && c.stages == stages && c.splits == splits)
                return c.ms;
        const float ms = make_and_time(tile, chunk, stages, splits);
        all.push_back({tile, chunk, stages, splits, ms});
        return ms;
    };
    for (int t : tiles) trial(t, 0, 0, 0);
    std::vector<Candidate> ranked;
    for (const Candidate &c : all)
        if (c.ms > 0) ranked.push_back(c);
    if (ranked.empty()) return set_error(BPGB_ERR_UNSUPPORTED, "no tile preset runs this workload");
    std::sort(ranked.begin(), ranked.end(),
              [](const Candidate &x, const Candidate &y) { return x.ms < y.ms; });
    const int top = std::min<int>(2, (int)ranked.size());
    for (int r = 0; r < top; r++)
        for (int chunk : {16, 32, 64})
            for (int stages : {2, 3, 4}) trial(ranked[r].tile, chunk, stages, 0);
    auto fastest = [&]() {
        std::vector<Candidate> ok;
        for (const Candidate &c : all)
            if (c.ms > 0) ok.push_back(c);
        std::sort(ok.begin(), ok.end(),
                  [](const Candidate &x, const Candidate &y) { return x.ms < y.ms; });
        return ok;
    };
    if (try_splits) {
        const Candidate w = fastest().front();
        for (int sp : {1, 2, 4}) trial(w.tile, w.chunk, w.stages, sp);
    }
    const std::vector<Candidate> order = fastest();
    for (const Candidate &c : order) {
        if (!validate(c.tile, c.chunk, c.stages, c.splits)) continue;
        best->tile = c.tile;
        best->chunk = c.chunk;
        best->stages = c.stages;
        best->splits = c.splits;
        best->ms = c.ms;
        if (rep) {
            rep->candidates = (uint32_t)all.size();
            rep->best_ms = c.ms;
            rep->default_ms = -1.0f;
            for (const Candidate &d : all)
                if (d.tile == tiles.front() && d.chunk == 0 && d.stages == 0 && d.splits == 0)
                    rep->default_ms = d.ms;
        }
        return BPGB_OK;
    }
    return set_error(BPGB_ERR_WINDOW, "every tuned candidate put bins outside their windows");
}

void fill(bpgb_options *opt, const TuneEntry &e, bpgb_tune_report *rep, bool hit) {
    opt->tile = e.tile;
    opt->chunk = e.chunk;
    opt->stages = e.stages;
    opt->pair_splits = e.splits;
    if (rep) {
        rep->cache_hit = hit ? 1 : 0;
        rep->tile = e.tile;
        rep->chunk = e.chunk;
        rep->stages = e.stages;
        rep->pair_splits = e.splits;
        if (hit) {
            rep->candidates = 0;
            rep->best_ms = e.ms;
            rep->default_ms = -1.0f;
        }
    }
}

bool lookup(const std::string &key, TuneEntry *e) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) return false;
    *e = it->second;
    return true;
}

void store(const std::string &key, const TuneEntry &e) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[key] = e;
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" {

int bpgb_plan_autotune(const bpgb_pair *host_pairs, uint64_t num_pairs, uint32_t T,
                       const uint32_t *voxels_per_side, const float *volume_zero_pos,
                       const float *voxel_inc, float t0, float deltaT, const void *d_H,
                       void *d_volume, bpgb_options *opt, bpgb_tune_report *report,
                       void *stream) {
    clear_error();
    if (!host_pairs || !voxels_per_side || !volume_zero_pos || !voxel_inc || !d_H || !d_volume ||
        !opt)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    if (report) std::memset(report, 0, sizeof(*report));
    int st = require_device();
    if (st) return st;
    bpgb_options base = *opt;
    base.algo = BPGB_ALGO_FAST;
    base.checked = 0;
    std::ostringstream k;
    k << "plan/" << device_tag() << "/dt" << base.h_dtype << "/acc" << base.accum << "/P"
      << num_pairs << "/T" << T << "/n" << voxels_per_side[0] << "x" << voxels_per_side[1] << "x"
      << voxels_per_side[2] << "/dT" << deltaT << "/pitch" << (base.h_pitch ? base.h_pitch : T);
    if (base.unfactored) k << "/unfactored";
    const std::string key = k.str();
    TuneEntry e;
    if (lookup(key, &e)) {
        fill(opt, e, report, true);
        opt->algo = BPGB_ALGO_FAST;
        return BPGB_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    auto make = [&](int tile, int chunk, int stages, int splits, int checked, bpgb_plan *out) {
        bpgb_options o = base;
        o.tile = tile;
        o.chunk = chunk;
        o.stages = stages;
        o.pair_splits = splits;
        o.checked = checked;
        return bpgb_plan_create(out, host_pairs, num_pairs, T, voxels_per_side, volume_zero_pos,
                                voxel_inc, t0, deltaT, &o);
    };
    auto make_and_time = [&](int tile, int chunk, int stages, int splits) {
        bpgb_plan p = nullptr;
        if (make(tile, chunk, stages, splits, 0, &p)) return -1.0f;
        const float ms = time_candidate([&]() { return bpgb_plan_execute(p, d_H, d_volume, s); }, s);
        bpgb_plan_destroy(p);
        return ms;
    };
    auto validate = [&](int tile, int chunk, int stages, int splits) {
        bpgb_plan p = nullptr;
        if (make(tile, chunk, stages, splits, 1, &p)) return false;
        uint64_t viol = 1;
        const bool ok = bpgb_plan_execute(p, d_H, d_volume, s) == 0 &&
                        bpgb_plan_check(p, &viol) == 0 && viol == 0;
        bpgb_plan_destroy(p);
        return ok;
    };
    std::vector<int> tiles;
    for (int t = 0; t < fast_preset_count(); t++) tiles.push_back(t);
    st = search(tiles, true, make_and_time, validate, &e, report);
    clear_error();
    if (st) return set_error(st, "autotune found no runnable configuration");
    store(key, e);
    fill(opt, e, report, false);
    opt->algo = BPGB_ALGO_FAST;
    return BPGB_OK;
}

int bpgb_batch_autotune(const bpgb_capture_geometry *captures, uint32_t n, const void *d_H,
                        float *d_volumes, bpgb_options *opt, bpgb_tune_report *report,
                        void *stream) {
    clear_error();
    if (!captures || !n || !d_H || !d_volumes || !opt)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    if (report) std::memset(report, 0, sizeof(*report));
    int st = require_device();
    if (st) return st;
    bpgb_options base = *opt;
    base.checked = 0;
    // shape signature of the batch (FNV-1a over the per-capture shapes)
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int b = 0; b < 8; b++) {
            h ^= (v >> (8 * b)) & 0xff;
            h *= 1099511628211ull;
        }
    };
    for (uint32_t c = 0; c < n; c++) {
        mix(captures[c].num_pairs);
        mix(captures[c].T);
        for (int a = 0; a < 3; a++) mix(captures[c].voxels_per_side[a]);
        uint32_t dT;
        std::memcpy(&dT, &captures[c].deltaT, 4);
        mix(dT);
    }
    std::ostringstream k;
    k << "batch/" << device_tag() << "/dt" << base.h_dtype << "/n" << n << "/shape" << std::hex << h;
    const std::string key = k.str();
    TuneEntry e;
    if (lookup(key, &e)) {
        fill(opt, e, report, true);
        return BPGB_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    auto make = [&](int tile, int chunk, int stages, int checked, bpgb_batch *out) {
        bpgb_options o = base;
        o.tile = tile;
        o.chunk = chunk;
        o.stages = stages;
        o.checked = checked;
        return bpgb_batch_create(out, captures, n, &o);
    };
    auto make_and_time = [&](int tile, int chunk, int stages, int) {
        bpgb_batch b = nullptr;
        if (make(tile, chunk, stages, 0, &b)) return -1.0f;
        const float ms =
            time_candidate([&]() { return bpgb_batch_execute(b, d_H, d_volumes, s); }, s);
        bpgb_batch_destroy(b);
        return ms;
    };
    auto validate = [&](int tile, int chunk, int stages, int) {
        bpgb_batch b = nullptr;
        if (make(tile, chunk, stages, 1, &b)) return false;
        uint64_t viol = 1;
        const bool ok = bpgb_batch_execute(b, d_H, d_volumes, s) == 0 &&
                        bpgb_batch_check(b, &viol) == 0 && viol == 0;
        bpgb_batch_destroy(b);
        return ok;
    };
    std::vector<int> tiles;
    for (int t = 0; t < fast_preset_count(); t++)
        if (fast_preset(t, base.h_dtype).k == 8 && fast_preset(t, base.h_dtype).consumer_warps() == 8 &&
            fast_preset(t, base.h_dtype).groups == 1)
            tiles.push_back(t);
    st = search(tiles, false, make_and_time, validate, &e, report);
    clear_error();
    if (st) return set_error(st, "autotune found no runnable configuration");
    store(key, e);
    fill(opt, e, report, false);
    return BPGB_OK;
}

int bpgb_tune_cache_clear(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache.clear();
    return BPGB_OK;
}

int bpgb_tune_cache_save(const char *path) {
    clear_error();
    if (!path) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null path");
    std::lock_guard<std::mutex> lock(g_mu);
    std::ofstream f(path, std::ios::trunc);
    if (!f) return set_error(BPGB_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    for (const auto &kv : g_cache)
        f << kv.first << ' ' << kv.second.tile << ' ' << kv.second.chunk << ' '
          << kv.second.stages << ' ' << kv.second.splits << ' ' << kv.second.ms << '\n';
    return f ? BPGB_OK : set_error(BPGB_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
}

int bpgb_tune_cache_load(const char *path) {
    clear_error();
    if (!path) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null path");
    std::ifstream f(path);
    if (!f) return BPGB_OK;  // no cache yet
    std::string line;
    int lineno = 0;
    std::map<std::string, TuneEntry> read;
    while (std::getline(f, line)) {
        lineno++;
        if (line.empty()) continue;
        std::istringstream in(line);
        std::string key;
        TuneEntry e;
        if (!(in >> key >> e.tile >> e.chunk >> e.stages >> e.splits >> e.ms) ||
            e.tile < -1 || e.tile >= fast_preset_count() || e.chunk < 0 || e.chunk > 64 ||
            e.stages < 0 || e.stages > 8 || e.splits < 0)
            return set_error(BPGB_ERR_INVALID_ARGUMENT,
                             std::string(path) + ":" + std::to_string(lineno) + ": bad entry");
        read[key] = e;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    for (const auto &kv : read) g_cache[kv.first] = kv.second;
    return BPGB_OK;
}

int bpgb_tune_cache_size(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    return (int)g_cache.size();
}

}  // extern "C"
