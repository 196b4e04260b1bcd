// C ABI: errors, plans (geometry analysis + algorithm selection), execute, and the
// drop-in host-buffer calls that replace call_cuda_backprojection /
// call_cuda_complex_backprojection (backproject_cuda.cu:370-500, 671-801).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "bpgb_internal.h"

namespace bpgb {

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
}  // namespace

int set_error(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

void clear_error() { g_last_error.clear(); }

int cuda_error(cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_error(BPGB_ERR_OUT_OF_MEMORY, m);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return set_error(BPGB_ERR_NO_DEVICE, m);
    return set_error(BPGB_ERR_CUDA, m);
}

void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int require_device(int *sm_count) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    int major = 0, sms = 0;
    e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaDeviceGetAttribute");
    if (major != 10)
        return set_error(BPGB_ERR_NO_DEVICE,
                         "this build targets sm_103a (GB300); device major version " +
                             std::to_string(major));
    if (sm_count) *sm_count = sms;
    return BPGB_OK;
}

EncodeTiledFn tensor_map_encoder() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

int reserve_dynamic_smem(const void *kernel, uint32_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, uint32_t> limits;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    uint32_t &cur = limits[{dev, kernel}];
    if (bytes <= cur) return BPGB_OK;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(max dynamic shared memory)");
    cur = bytes;
    return BPGB_OK;
}

namespace {

// The host drop-in call's plan of the last geometry it saw, keyed by every input the
// plan depends on (the pairs compared byte for byte).
struct HostPlanCache {
    bpgb_plan plan = nullptr;
    std::vector<bpgb_pair> pairs;
    std::vector<unsigned char> key;

    static std::vector<unsigned char> make_key(uint64_t num_pairs, uint32_t T, const uint32_t *n,
                                               const float *zero, const float *inc, float t0,
                                               float deltaT, const bpgb_options &o) {
        std::vector<unsigned char> k;
        auto put = [&](const void *p, size_t b) {
            const unsigned char *c = (const unsigned char *)p;
            k.insert(k.end(), c, c + b);
        };
        const float none[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        put(&num_pairs, sizeof num_pairs);
        put(&T, sizeof T);
        put(n, 3 * sizeof(uint32_t));
        put(zero ? zero : none, 3 * sizeof(float));
        put(inc ? inc : none, 9 * sizeof(float));
        put(&t0, sizeof t0);
        put(&deltaT, sizeof deltaT);
        put(&o, sizeof o);
        return k;
    }
    bpgb_plan find(const bpgb_pair *p, uint64_t np, uint32_t T, const uint32_t *n,
                   const float *zero, const float *inc, float t0, float deltaT,
                   const bpgb_options &o) const {
        if (!plan || pairs.size() != np) return nullptr;
        if (make_key(np, T, n, zero, inc, t0, deltaT, o) != key) return nullptr;
        if (np && std::memcmp(pairs.data(), p, np * sizeof(bpgb_pair)) != 0) return nullptr;
        return plan;
    }
    void keep(bpgb_plan pl, const bpgb_pair *p, uint64_t np, uint32_t T, const uint32_t *n,
              const float *zero, const float *inc, float t0, float deltaT,
              const bpgb_options &o) {
        plan = pl;
        pairs.assign(p, p + np);
        key = make_key(np, T, n, zero, inc, t0, deltaT, o);
    }
    void clear() {
        if (plan) bpgb_plan_destroy(plan);
        plan = nullptr;
        pairs.clear();
        key.clear();
    }
    ~HostPlanCache() { clear(); }
};

}  // namespace

int DeviceBuffer::reserve(size_t need) {
    if (need <= bytes) return BPGB_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, need);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return cuda_error(e, "cudaMalloc");
    }
    bytes = need;
    return BPGB_OK;
}

DeviceBuffer::~DeviceBuffer() {
    // Process teardown may run after the CUDA context is gone; freeing then is harmless.
    if (ptr) cudaFree(ptr);
}

static bool same3(const float *a, const float *b) {
    return std::memcmp(a, b, 3 * sizeof(float)) == 0;
}

Factorization factorize_pairs(const bpgb_pair *pairs, uint64_t P) {
    Factorization f;
    f.L = P;
    f.S = 1;
    if (P == 0) return f;
    // Confocal (precompute_distances, backproject.hpp:399-413): laser point == camera
    // point and equal legs for every pair.
    bool confocal = true;
    for (uint64_t p = 0; p < P && confocal; p++)
        confocal = same3(pairs[p].laser_point, pairs[p].camera_point) &&
                   pairs[p].laser_wall == pairs[p].camera_wall;
    if (confocal && P > 1) {
        f.geom = GEOM_CONFOCAL;
        f.L = 1;
        f.S = P;
        return f;
    }
    // Exhaustive order p = l * S + s (backproject.hpp:386-389): S = run length of the
    // first laser point, then every block repeats the first block's SPAD list.
    uint64_t S = 1;
    while (S < P && same3(pairs[S].laser_point, pairs[0].laser_point) &&
           pairs[S].laser_wall == pairs[0].laser_wall)
        S++;
    if (P % S != 0) return f;
    const uint64_t L = P / S;
    for (uint64_t l = 0; l < L; l++) {
        const bpgb_pair &head = pairs[l * S];
        for (uint64_t s = 0; s < S; s++) {
            const bpgb_pair &q = pairs[l * S + s];
            if (!same3(q.laser_point, head.laser_point) || q.laser_wall != head.laser_wall ||
                !same3(q.camera_point, pairs[s].camera_point) ||
                q.camera_wall != pairs[s].camera_wall)
                return f;
        }
        if (l > 0 && same3(head.laser_point, pairs[0].laser_point)) return f;
    }
    if (S == 1) return f;  // one SPAD per laser: nothing to factor
    f.geom = L == 1 ? GEOM_SINGLE_LASER : GEOM_EXHAUSTIVE;
    f.L = L;
    f.S = S;
    return f;
}

bool volume_frame(const Volume &vol, double u[3][3], double h[3]) {
    for (int a = 0; a < 3; a++) {
        double n2 = 0.0;
        for (int k = 0; k < 3; k++) n2 += (double)vol.inc[3 * a + k] * vol.inc[3 * a + k];
        h[a] = std::sqrt(n2);
        if (!(h[a] > 0.0) || !std::isfinite(h[a])) return false;
        for (int k = 0; k < 3; k++) u[a][k] = vol.inc[3 * a + k] / h[a];
    }
    for (int a = 0; a < 3; a++)
        for (int b = a + 1; b < 3; b++) {
            double d = 0.0;
            for (int k = 0; k < 3; k++) d += u[a][k] * u[b][k];
            if (std::fabs(d) > 1e-5) return false;
        }
    return true;
}

bool finite_geometry(const bpgb_pair *pairs, uint64_t P, const Volume &vol,
                            const BinParams &bp, std::string *why) {
    for (uint64_t p = 0; p < P; p++) {
        const float *f = reinterpret_cast<const float *>(&pairs[p]);
        for (int k = 0; k < 8; k++)
            if (!std::isfinite(f[k])) {
                *why = "pair " + std::to_string(p) + " has a non-finite coordinate or leg";
                return false;
            }
    }
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(vol.zero[k])) {
            *why = "volume_zero_pos is not finite";
            return false;
        }
    for (int k = 0; k < 9; k++)
        if (!std::isfinite(vol.inc[k])) {
            *why = "voxel_inc is not finite";
            return false;
        }
    if (!std::isfinite(bp.t0) || !std::isfinite(bp.dT) || bp.dT == 0.0f) {
        *why = "t0 / deltaT must be finite and deltaT non-zero";
        return false;
    }
    return true;
}

}  // namespace bpgb

using namespace bpgb;

struct bpgb_plan_s {
    int algo = BPGB_ALGO_EXACT;
    bpgb_options opt{};
    Volume vol{};
    BinParams bp{};
    uint64_t P = 0;
    Factorization fz{};
    bpgb_pair *d_pairs = nullptr;
    FastPlan *fast = nullptr;
    cudaStream_t last_stream = nullptr;
};

extern "C" {

int bpgb_abi_version(void) { return BPGB_ABI_VERSION; }

const char *bpgb_status_string(int status) {
    switch (status) {
        case BPGB_OK: return "ok";
        case BPGB_ERR_INVALID_ARGUMENT: return "invalid argument";
        case BPGB_ERR_CUDA: return "CUDA error";
        case BPGB_ERR_OUT_OF_MEMORY: return "out of device memory";
        case BPGB_ERR_TIMEOUT: return "device wait timed out";
        case BPGB_ERR_UNSUPPORTED: return "unsupported by the selected algorithm";
        case BPGB_ERR_NO_DEVICE: return "no GB300 device";
        case BPGB_ERR_WINDOW: return "bin outside its staged window";
    }
    return "unknown status";
}

const char *bpgb_last_error(void) { return g_last_error.c_str(); }

uint64_t bpgb_launch_count(void) { return g_launches.load(); }

void bpgb_options_default(bpgb_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->algo = BPGB_ALGO_AUTO;
    opt->h_dtype = BPGB_DTYPE_F32;
    opt->accum = BPGB_ACCUM_F32;
    opt->h_scale = 1.0f;
    opt->tile = -1;
}

int bpgb_plan_create(bpgb_plan *plan, const bpgb_pair *host_pairs, uint64_t num_pairs,
                     uint32_t T, const uint32_t *voxels_per_side, const float *volume_zero_pos,
                     const float *voxel_inc, float t0, float deltaT, const bpgb_options *opt) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    *plan = nullptr;
    if (!voxels_per_side || !volume_zero_pos || !voxel_inc)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "volume description is null");
    if (num_pairs > 0 && !host_pairs)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "host_pairs is null");
    if (T == 0) return set_error(BPGB_ERR_INVALID_ARGUMENT, "T must be positive");
    bpgb_options o;
    bpgb_options_default(&o);
    if (opt) o = *opt;
    if (o.h_dtype < BPGB_DTYPE_F32 || o.h_dtype > BPGB_DTYPE_C32)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "unknown h_dtype");
    if (o.h_pitch && o.h_pitch < T) return set_error(BPGB_ERR_INVALID_ARGUMENT, "h_pitch < T");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;

    auto *p = new bpgb_plan_s();
    p->opt = o;
    for (int k = 0; k < 3; k++) {
        p->vol.n[k] = voxels_per_side[k];
        p->vol.zero[k] = volume_zero_pos[k];
    }
    for (int k = 0; k < 9; k++) p->vol.inc[k] = voxel_inc[k];
    p->bp.t0 = t0;
    p->bp.dT = deltaT;
    p->bp.T = T;
    p->P = num_pairs;
    std::string why;
    if (!finite_geometry(host_pairs, num_pairs, p->vol, p->bp, &why)) {
        delete p;
        return set_error(BPGB_ERR_INVALID_ARGUMENT, why);
    }
    if (num_pairs) {
        cudaError_t e = cudaMalloc(&p->d_pairs, num_pairs * sizeof(bpgb_pair));
        if (e == cudaSuccess)
            e = cudaMemcpy(p->d_pairs, host_pairs, num_pairs * sizeof(bpgb_pair),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            bpgb_plan_destroy(p);
            return cuda_error(e, "plan pair upload");
        }
    }
    p->fz = factorize_pairs(host_pairs, num_pairs);
    const bool low_precision = o.h_dtype == BPGB_DTYPE_F16 || o.h_dtype == BPGB_DTYPE_BF16 ||
                               o.h_dtype == BPGB_DTYPE_C32;
    int algo = o.algo;
    if (algo == BPGB_ALGO_AUTO || algo == BPGB_ALGO_FAST || low_precision ||
        o.accum == BPGB_ACCUM_KAHAN) {
        if (algo == BPGB_ALGO_EXACT && (low_precision || o.accum == BPGB_ACCUM_KAHAN)) {
            bpgb_plan_destroy(p);
            return set_error(BPGB_ERR_UNSUPPORTED,
                             "EXACT computes FP32/complex64 rows with FP32 sums only");
        }
        why.clear();
        st = num_pairs ? fast_plan_build(&p->fast, p->d_pairs, num_pairs, p->fz,
                                         p->vol, p->bp, o, sms, &why)
                       : BPGB_ERR_UNSUPPORTED;
        if (st == BPGB_OK) {
            algo = BPGB_ALGO_FAST;
        } else if (st == BPGB_ERR_UNSUPPORTED && o.algo == BPGB_ALGO_AUTO && !low_precision &&
                   o.accum != BPGB_ACCUM_KAHAN) {
            algo = BPGB_ALGO_EXACT;
            clear_error();
        } else {
            bpgb_plan_destroy(p);
            if (st == BPGB_ERR_UNSUPPORTED) return set_error(st, "FAST path: " + why);
            return st;
        }
    }
    p->algo = algo;
    *plan = p;
    return BPGB_OK;
}

int bpgb_plan_execute(bpgb_plan plan, const void *d_H, void *d_volume, void *stream) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    if (!d_volume) return set_error(BPGB_ERR_INVALID_ARGUMENT, "d_volume is null");
    if (plan->P && !d_H) return set_error(BPGB_ERR_INVALID_ARGUMENT, "d_H is null");
    cudaStream_t s = (cudaStream_t)stream;
    plan->last_stream = s;
    const bool cplx = plan->opt.h_dtype == BPGB_DTYPE_C64 || plan->opt.h_dtype == BPGB_DTYPE_C32;
    if (plan->P == 0) {
        BPGB_CUDA_TRY(cudaMemsetAsync(d_volume, 0, plan->vol.count() * (cplx ? 8 : 4), s));
        return BPGB_OK;
    }
    if (plan->algo == BPGB_ALGO_FAST) return fast_plan_execute(plan->fast, d_H, d_volume, s);
    const uint64_t pitch = plan->opt.h_pitch ? plan->opt.h_pitch : plan->bp.T;
    int st = launch_exact(d_H, cplx, pitch, plan->d_pairs, plan->P, plan->vol, plan->bp,
                          d_volume, s);
    if (st) return st;
    if (plan->opt.h_scale != 1.0f && plan->opt.h_scale != 0.0f)
        return set_error(BPGB_ERR_UNSUPPORTED, "h_scale applies to the FAST path only");
    return BPGB_OK;
}

int bpgb_plan_execute_tiles(bpgb_plan plan, const void *d_H, void *d_volume,
                            const uint32_t *d_tile_list, const uint32_t *d_tile_count,
                            uint32_t max_tiles, void *stream) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    if (!d_volume || !d_H) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null buffer");
    if (plan->algo != BPGB_ALGO_FAST || !plan->fast)
        return set_error(BPGB_ERR_UNSUPPORTED, "tile-list launches need a FAST plan");
    cudaStream_t s = (cudaStream_t)stream;
    plan->last_stream = s;
    return fast_plan_execute_tiles(plan->fast, d_H, d_volume, d_tile_list, d_tile_count,
                                   max_tiles, s);
}

int bpgb_plan_select_tiles(bpgb_plan plan, const float *d_block_score,
                           const uint32_t *block_dims, uint32_t block_size, float threshold,
                           uint32_t *d_tile_list, uint32_t *d_tile_count, void *stream) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    if (plan->algo != BPGB_ALGO_FAST || !plan->fast)
        return set_error(BPGB_ERR_UNSUPPORTED, "tile selection needs a FAST plan");
    return fast_plan_select_tiles(plan->fast, d_block_score, block_dims, block_size, threshold,
                                  d_tile_list, d_tile_count, (cudaStream_t)stream);
}

int bpgb_plan_select_tiles_topk(bpgb_plan plan, const float *d_block_score,
                                const uint32_t *block_dims, uint32_t block_size, uint32_t k,
                                uint32_t *d_tile_list, uint32_t *d_tile_count, void *stream) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    if (plan->algo != BPGB_ALGO_FAST || !plan->fast)
        return set_error(BPGB_ERR_UNSUPPORTED, "tile selection needs a FAST plan");
    return fast_plan_select_tiles_topk(plan->fast, d_block_score, block_dims, block_size, k,
                                       d_tile_list, d_tile_count, (cudaStream_t)stream);
}

int bpgb_plan_check(bpgb_plan plan, uint64_t *violations) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    BPGB_CUDA_TRY(cudaStreamSynchronize(plan->last_stream));
    if (violations) *violations = 0;
    if (plan->algo != BPGB_ALGO_FAST) return BPGB_OK;
    uint64_t v = 0, t = 0;
    int st = fast_plan_check(plan->fast, &v, &t);
    if (st) return st;
    if (violations) *violations = v;
    if (t) return set_error(BPGB_ERR_TIMEOUT, std::to_string(t) + " device waits timed out");
    if (v) return set_error(BPGB_ERR_WINDOW, std::to_string(v) + " bins fell outside their window");
    return BPGB_OK;
}

int bpgb_plan_get_info(bpgb_plan plan, bpgb_plan_info *info) {
    if (!plan || !info) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->updates = plan->vol.count() * plan->P;
    if (plan->algo == BPGB_ALGO_FAST) {
        fast_plan_info(plan->fast, info);
        info->updates = plan->vol.count() * plan->P;
        return BPGB_OK;
    }
    info->algo = BPGB_ALGO_EXACT;
    info->geometry = plan->fz.geom;
    info->num_lasers = plan->fz.L;
    info->num_spads = plan->fz.S;
    info->tile[0] = 4;
    info->tile[1] = 8;
    info->tile[2] = 8;
    info->pair_splits = 1;
    info->grid = (uint32_t)(((plan->vol.n[0] + 3) / 4) * ((plan->vol.n[1] + 7) / 8) *
                            ((plan->vol.n[2] + 7) / 8));
    info->threads = 256;
    info->scratch_bytes = plan->P * sizeof(bpgb_pair);
    return BPGB_OK;
}

int bpgb_plan_dump_bins(bpgb_plan plan, const int64_t *h_voxel_ids, int64_t n, int32_t *d_bins,
                        void *stream) {
    clear_error();
    if (!plan || (n > 0 && (!h_voxel_ids || !d_bins)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    if (n <= 0) return BPGB_OK;
    const uint64_t nvox = plan->vol.count();
    for (int64_t i = 0; i < n; i++)
        if (h_voxel_ids[i] < 0 || (uint64_t)h_voxel_ids[i] >= nvox)
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "voxel id out of range");
    cudaStream_t s = (cudaStream_t)stream;
    int64_t *d_ids = nullptr;
    BPGB_CUDA_TRY(cudaMalloc(&d_ids, n * sizeof(int64_t)));
    cudaError_t e = cudaMemcpy(d_ids, h_voxel_ids, n * sizeof(int64_t), cudaMemcpyHostToDevice);
    int st = BPGB_OK;
    if (e != cudaSuccess) {
        st = cuda_error(e, "voxel id upload");
    } else if (plan->algo == BPGB_ALGO_FAST) {
        st = fast_plan_dump_bins(plan->fast, d_ids, n, d_bins, s);
    } else {
        st = launch_exact_bins(plan->d_pairs, plan->P, plan->vol, plan->bp, d_ids, n, d_bins, s);
    }
    e = cudaStreamSynchronize(s);
    cudaFree(d_ids);
    if (st) return st;
    if (e != cudaSuccess) return cuda_error(e, "dump bins");
    return BPGB_OK;
}

int bpgb_plan_get_tables(bpgb_plan plan, float *host_out, uint64_t capacity,
                         uint64_t *num_entries) {
    clear_error();
    if (!plan) return set_error(BPGB_ERR_INVALID_ARGUMENT, "plan is null");
    if (plan->algo != BPGB_ALGO_FAST || !plan->fast)
        return set_error(BPGB_ERR_UNSUPPORTED, "tables belong to FAST plans");
    return fast_plan_tables(plan->fast, host_out, capacity, num_entries);
}

int bpgb_plan_destroy(bpgb_plan plan) {
    if (!plan) return BPGB_OK;
    if (plan->fast) fast_plan_free(plan->fast);
    if (plan->d_pairs) cudaFree(plan->d_pairs);
    delete plan;
    return BPGB_OK;
}

int bpgb_diag_wait_timeout(uint32_t spin_limit) {
    clear_error();
    int st = require_device();
    if (st) return st;
    int timed_out = 0;
    st = wait_timeout_probe(spin_limit ? spin_limit : 1, &timed_out);
    if (st) return st;
    if (timed_out)
        return set_error(BPGB_ERR_TIMEOUT, "probe wait gave up after " + std::to_string(spin_limit) +
                                               " polls");
    return BPGB_OK;
}

// ---- drop-in host-buffer calls --------------------------------------------------

int bpgb_backproject_host(const void *transient_chunk, uint64_t transient_size, uint32_t T,
                          const bpgb_pair *scanned_pairs, uint64_t num_pairs,
                          void *voxel_volume, const uint32_t *voxels_per_side,
                          const float *volume_zero_pos, const float *voxel_inc, float t0,
                          float deltaT, const bpgb_options *opt) {
    clear_error();
    bpgb_options o;
    bpgb_options_default(&o);
    if (opt) o = *opt;
    if (!voxel_volume || !voxels_per_side)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "voxel_volume / voxels_per_side is null");
    if (T == 0) return set_error(BPGB_ERR_INVALID_ARGUMENT, "T must be positive");
    if (transient_size != num_pairs * (uint64_t)T)
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "transient_size must equal num_pairs * T (" +
                             std::to_string(transient_size) + " != " +
                             std::to_string(num_pairs) + " * " + std::to_string(T) + ")");
    if (num_pairs && !transient_chunk)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "transient_chunk is null");
    const int dt = o.h_dtype;
    const size_t esz = dt == BPGB_DTYPE_C64 ? 8 : (dt == BPGB_DTYPE_F32 || dt == BPGB_DTYPE_C32 ? 4 : 2);
    const size_t out_esz = dt == BPGB_DTYPE_C64 || dt == BPGB_DTYPE_C32 ? 8 : 4;
    // Rows are copied into a 16-byte aligned pitch so the TMA path applies to any T.
    const uint32_t align = (uint32_t)(16 / esz);
    const uint32_t pitch = (T + align - 1) / align * align;
    o.h_pitch = pitch;

    // Repeated calls on one scan geometry (new transient data, same pairs, grid, t0, deltaT
    // and options) reuse the calling thread's last plan instead of rebuilding its tables.
    thread_local HostPlanCache cache;
    bpgb_plan plan = cache.find(scanned_pairs, num_pairs, T, voxels_per_side, volume_zero_pos,
                                voxel_inc, t0, deltaT, o);
    int st = BPGB_OK;
    if (!plan) {
        cache.clear();
        st = bpgb_plan_create(&plan, scanned_pairs, num_pairs, T, voxels_per_side,
                              volume_zero_pos, voxel_inc, t0, deltaT, &o);
        if (st) return st;
        cache.keep(plan, scanned_pairs, num_pairs, T, voxels_per_side, volume_zero_pos, voxel_inc,
                   t0, deltaT, o);
    }
    const uint64_t nvox = (uint64_t)voxels_per_side[0] * voxels_per_side[1] * voxels_per_side[2];
    thread_local DeviceBuffer dH, dV;
    st = dH.reserve(std::max<size_t>(16, num_pairs * (size_t)pitch * esz));
    if (!st) st = dV.reserve(std::max<size_t>(16, nvox * out_esz));
    if (!st && num_pairs) {
        cudaError_t e;
        if (pitch == T)
            e = cudaMemcpy(dH.ptr, transient_chunk, num_pairs * (size_t)T * esz,
                           cudaMemcpyHostToDevice);
        else
            e = cudaMemcpy2D(dH.ptr, pitch * esz, transient_chunk, (size_t)T * esz,
                             (size_t)T * esz, num_pairs, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) st = cuda_error(e, "H upload");
    }
    if (!st) st = bpgb_plan_execute(plan, dH.ptr, dV.ptr, nullptr);
    if (!st) st = bpgb_plan_check(plan, nullptr);
    if (!st) {
        cudaError_t e = cudaMemcpy(voxel_volume, dV.ptr, nvox * out_esz, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_error(e, "volume download");
    }
    if (st) {  // a failed call does not leave its plan for the next one
        const std::string keep(bpgb_last_error());
        cache.clear();
        set_error(st, keep);
    }
    return st;
}

}  // extern "C"

namespace {
// Algorithm of the drop-in calls (bpgb_backproject_f32 / _c64 and the call_cuda_* shim):
// BPGB_ALGO=exact|fast|auto in the environment at first use, bpgb_set_dropin_algo after.
std::atomic<int> g_dropin_algo{-1};

int dropin_algo() {
    int a = g_dropin_algo.load(std::memory_order_relaxed);
    if (a >= 0) return a;
    a = BPGB_ALGO_AUTO;
    if (const char *e = std::getenv("BPGB_ALGO")) {
        const std::string v(e);
        if (v == "exact" || v == "EXACT" || v == "1") a = BPGB_ALGO_EXACT;
        else if (v == "fast" || v == "FAST" || v == "2") a = BPGB_ALGO_FAST;
    }
    int expected = -1;
    g_dropin_algo.compare_exchange_strong(expected, a);
    return g_dropin_algo.load(std::memory_order_relaxed);
}
}  // namespace

extern "C" {

int bpgb_set_dropin_algo(int algo) {
    clear_error();
    if (algo != BPGB_ALGO_AUTO && algo != BPGB_ALGO_EXACT && algo != BPGB_ALGO_FAST)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "algo must be BPGB_ALGO_AUTO, _EXACT or _FAST");
    g_dropin_algo.store(algo, std::memory_order_relaxed);
    return BPGB_OK;
}

int bpgb_get_dropin_algo(void) { return dropin_algo(); }

int bpgb_backproject_f32(const float *transient_chunk, uint64_t transient_size, uint32_t T,
                         const bpgb_pair *scanned_pairs, uint64_t num_pairs,
                         float *voxel_volume, const uint32_t *voxels_per_side,
                         const float *volume_zero_pos, const float *voxel_inc, float t0,
                         float deltaT) {
    bpgb_options o;
    bpgb_options_default(&o);
    o.algo = dropin_algo();
    o.h_dtype = BPGB_DTYPE_F32;
    return bpgb_backproject_host(transient_chunk, transient_size, T, scanned_pairs, num_pairs,
                                 voxel_volume, voxels_per_side, volume_zero_pos, voxel_inc, t0,
                                 deltaT, &o);
}

int bpgb_backproject_c64(const float *transient_chunk, uint64_t transient_size, uint32_t T,
                         const bpgb_pair *scanned_pairs, uint64_t num_pairs,
                         float *voxel_volume, const uint32_t *voxels_per_side,
                         const float *volume_zero_pos, const float *voxel_inc, float t0,
                         float deltaT) {
    bpgb_options o;
    bpgb_options_default(&o);
    o.algo = dropin_algo();
    o.h_dtype = BPGB_DTYPE_C64;
    return bpgb_backproject_host(transient_chunk, transient_size, T, scanned_pairs, num_pairs,
                                 voxel_volume, voxels_per_side, volume_zero_pos, voxel_inc, t0,
                                 deltaT, &o);
}

}  // extern "C"
