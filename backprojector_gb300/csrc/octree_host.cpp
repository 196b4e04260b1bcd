// Learned-octree reconstruction as a native object (bpgb_octree_*): the coarse FAST pass,
// the occupancy CNN, the trilinear fill, tile selection and the block-sparse fine pass,
// queued on one stream from the public kernels of this library.  It replaces the
// reference's octree entry (call_cuda_octree_backprojection, backproject_cuda.hpp:30-39;
// backproject_cuda.cu:503-669) for callers that do not go through Python.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "bpgb_internal.h"
#include "npy.h"

using namespace bpgb;

namespace {

constexpr uint32_t kBlock = 8;
constexpr float kHTarget = 16384.0f;  // FP16 rows: max |H| maps here

struct Layer {
    uint32_t cin, cout, np;
    bool relu;
};

}  // namespace

struct bpgb_octree_s {
    uint32_t fine[3] = {0, 0, 0}, coarse[3] = {0, 0, 0}, tile[3] = {0, 0, 0};
    uint32_t tiles = 0, in_channels = 2, pair_splits = 8;
    uint64_t P = 0;
    uint32_t T = 0, pitch16 = 0;
    int h_dtype = BPGB_DTYPE_F16;
    float p_lo = 0.5f, logit_lo = 0.0f;
    bpgb_plan coarse_plan = nullptr, sparse_plan = nullptr;
    std::vector<Layer> layers;
    std::vector<void *> wt;  // packed BF16 weights per layer (mma.sync kernels)
    // tensor-core path (coarse grids of 32-voxel z-lines): FP32 masters (bias rows), the
    // tcgen05 weight images and the line-planes activations (padding rows zero)
    bool tc = false;
    std::vector<float *> master;
    std::vector<void *> wtc;
    void *Xl = nullptr, *Yl[3] = {nullptr, nullptr, nullptr};
    void *rows = nullptr;    // FP16 rows (FP16 mode)
    float *absmax = nullptr, *coarse_vol = nullptr, *logits = nullptr, *feat = nullptr;
    void *X = nullptr, *Y[3] = {nullptr, nullptr, nullptr};
    uint32_t *tile_list = nullptr, *tile_count = nullptr;
    uint64_t scratch = 0;
    cudaStream_t last = nullptr;
    float *io_H = nullptr, *io_vol = nullptr;  // device copies for the host-buffer call
};

namespace {

void octree_free(bpgb_octree_s *o) {
    if (!o) return;
    if (o->coarse_plan) bpgb_plan_destroy(o->coarse_plan);
    if (o->sparse_plan) bpgb_plan_destroy(o->sparse_plan);
    for (void *p : o->wt) cudaFree(p);
    for (float *p : o->master) cudaFree(p);
    for (void *p : o->wtc) cudaFree(p);
    cudaFree(o->Xl);
    for (void *p : o->Yl) cudaFree(p);
    cudaFree(o->rows);
    cudaFree(o->absmax);
    cudaFree(o->coarse_vol);
    cudaFree(o->logits);
    cudaFree(o->feat);
    cudaFree(o->X);
    for (void *p : o->Y) cudaFree(p);
    cudaFree(o->tile_list);
    cudaFree(o->tile_count);
    cudaFree(o->io_H);
    cudaFree(o->io_vol);
    delete o;
}

}  // namespace

extern "C" {

int bpgb_octree_create(bpgb_octree *out, const bpgb_pair *pairs, uint64_t num_pairs, uint32_t T,
                       const uint32_t *voxels_per_side, const float *volume_zero_pos,
                       const float *voxel_inc, float t0, float deltaT, const char *weights_path,
                       float p_lo, const bpgb_options *opt) {
    clear_error();
    if (!out || !pairs || !voxels_per_side || !volume_zero_pos || !voxel_inc || !weights_path)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    bpgb_options o;
    bpgb_options_default(&o);
    o.h_dtype = BPGB_DTYPE_F16;  // NULL opt: FP16 rows
    if (opt) o = *opt;
    if (o.h_dtype != BPGB_DTYPE_F32 && o.h_dtype != BPGB_DTYPE_F16)
        return set_error(BPGB_ERR_UNSUPPORTED, "the learned octree takes FP32 or FP16 rows");
    if (o.h_pitch && o.h_pitch != T)
        return set_error(BPGB_ERR_UNSUPPORTED, "the learned octree takes rows of pitch T");
    for (int k = 0; k < 3; k++)
        if (voxels_per_side[k] < 2 * kBlock || voxels_per_side[k] % kBlock)
            return set_error(BPGB_ERR_INVALID_ARGUMENT,
                             "voxels per side must be multiples of 8 and at least 16");
    std::map<std::string, NpyArray> w;
    std::string why;
    if (!npz_load(weights_path, &w, &why)) return set_error(BPGB_ERR_INVALID_ARGUMENT, why);
    auto *oc = new bpgb_octree_s();
    auto fail = [&](int st) {
        octree_free(oc);
        return st;
    };
    oc->in_channels = w.count("in_channels") ? (uint32_t)w["in_channels"].at(0) : 1u;
    if (oc->in_channels != 1 && oc->in_channels != 2)
        return fail(set_error(BPGB_ERR_INVALID_ARGUMENT, "weights: in_channels must be 1 or 2"));
    oc->p_lo = p_lo > 0.0f ? p_lo : (w.count("p_lo") ? (float)w["p_lo"].at(0) : 0.5f);
    if (!(oc->p_lo > 0.0f && oc->p_lo < 1.0f))
        return fail(set_error(BPGB_ERR_INVALID_ARGUMENT, "p_lo must lie in (0, 1)"));
    oc->logit_lo = std::log(oc->p_lo / (1.0f - oc->p_lo));
    oc->layers = {{oc->in_channels, 16, 16, true}, {16, 16, 16, true}, {16, 16, 16, true},
                  {16, 1, 8, false}};
    oc->P = num_pairs;
    oc->T = T;
    oc->h_dtype = o.h_dtype;
    oc->pair_splits = o.pair_splits > 0 ? (uint32_t)o.pair_splits : 8u;
    for (int k = 0; k < 3; k++) {
        oc->fine[k] = voxels_per_side[k];
        oc->coarse[k] = voxels_per_side[k] / kBlock;
    }
    // the coarse grid spans the same box: step x (n_fine - 1) / (n_coarse - 1)
    float inc_c[9];
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
            inc_c[3 * a + c] = (float)((double)voxel_inc[3 * a + c] * (oc->fine[a] - 1) /
                                       (double)(oc->coarse[a] - 1));
    if (o.h_dtype == BPGB_DTYPE_F16) oc->pitch16 = (T + 7) / 8 * 8;  // 16-byte FP16 rows
    bpgb_options po = o;
    po.algo = BPGB_ALGO_FAST;
    po.h_pitch = o.h_dtype == BPGB_DTYPE_F16 ? oc->pitch16 : 0;
    po.h_scale = 1.0f;
    po.checked = 0;
    po.tile = -1;
    po.pair_splits = 0;
    po.chunk = 0;
    po.stages = 0;
    int st = bpgb_plan_create(&oc->coarse_plan, pairs, num_pairs, T, oc->coarse, volume_zero_pos,
                              inc_c, t0, deltaT, &po);
    if (st) return fail(st);
    // 8^3 tiles = the CNN's blocks: four per CTA (preset 13) for plain sums, one per CTA
    // (preset 10) where the grouped form is not built (Kahan-compensated sums)
    po.tile = o.tile >= 0 ? o.tile : (o.accum == BPGB_ACCUM_KAHAN ? 10 : 13);
    po.pair_splits = (int32_t)oc->pair_splits;
    po.chunk = o.chunk;
    po.stages = o.stages;
    st = bpgb_plan_create(&oc->sparse_plan, pairs, num_pairs, T, oc->fine, volume_zero_pos,
                          voxel_inc, t0, deltaT, &po);
    if (st) return fail(st);
    bpgb_plan_info info;
    bpgb_plan_get_info(oc->sparse_plan, &info);
    oc->tiles = 1;
    for (int k = 0; k < 3; k++) {
        oc->tile[k] = info.tile[k];
        if (info.tile[k] % kBlock)
            return fail(set_error(BPGB_ERR_UNSUPPORTED, "fine tiles must be multiples of 8"));
        oc->tiles *= (oc->fine[k] + info.tile[k] - 1) / info.tile[k];
    }
    oc->scratch = info.scratch_bytes;
    // weights
    const uint64_t nc = (uint64_t)oc->coarse[0] * oc->coarse[1] * oc->coarse[2];
    cudaError_t e = cudaSuccess;
    oc->tc = oc->coarse[2] == 32 && oc->coarse[1] % 8 == 0;
    for (size_t li = 0; li < oc->layers.size(); li++) {
        const Layer &L = oc->layers[li];
        const std::string key = "w" + std::to_string(li);
        const uint32_t kp = bpgb_cnn_kp(L.cin);
        if (!w.count(key) || w[key].shape.size() != 2 || w[key].shape[0] != kp ||
            w[key].shape[1] != L.cout)
            return fail(set_error(BPGB_ERR_INVALID_ARGUMENT,
                                  "weights: " + key + " must be [" + std::to_string(kp) + ", " +
                                      std::to_string(L.cout) + "]"));
        const std::vector<float> m = w[key].as_float();
        float *d_m = nullptr;
        void *d_t = nullptr;
        e = cudaMalloc(&d_m, m.size() * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&d_t, (size_t)L.np * kp * 2);
        if (e == cudaSuccess)
            e = cudaMemcpy(d_m, m.data(), m.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (d_t) oc->wt.push_back(d_t);
        if (e == cudaSuccess) {
            st = bpgb_cnn_pack_weights(d_m, L.cin, L.cout, L.np, d_t, 0, nullptr, nullptr);
            if (st == 0 && oc->tc) {
                void *d_tc = nullptr;
                const uint64_t tb = bpgb_cnn_tc_weight_bytes(L.cin);
                e = cudaMalloc(&d_tc, tb);
                if (d_tc) oc->wtc.push_back(d_tc);
                if (e == cudaSuccess) st = bpgb_cnn_tc_pack_weights(d_m, L.cin, L.cout, d_tc, nullptr, nullptr);
                oc->scratch += tb + m.size() * sizeof(float);
            }
            if (st == 0 && e == cudaSuccess) e = cudaDeviceSynchronize();
        }
        if (oc->tc && d_m)
            oc->master.push_back(d_m);  // its bias row feeds the tensor-core epilogue
        else
            cudaFree(d_m);
        if (e != cudaSuccess) return fail(cuda_error(e, "octree weights"));
        if (st) return fail(st);
        oc->scratch += (uint64_t)L.np * kp * 2;
    }
    if (oc->tc) {
        const uint64_t xb = bpgb_cnn_lp_bytes(oc->in_channels, 0, oc->coarse, 1);
        const uint64_t yb = bpgb_cnn_lp_bytes(16, 0, oc->coarse, 1);
        e = cudaMalloc(&oc->Xl, xb);
        if (e == cudaSuccess) e = cudaMemset(oc->Xl, 0, xb);
        for (int k = 0; k < 3 && e == cudaSuccess; k++) {
            e = cudaMalloc(&oc->Yl[k], yb);
            if (e == cudaSuccess) e = cudaMemset(oc->Yl[k], 0, yb);
        }
        if (e != cudaSuccess) return fail(cuda_error(e, "octree line-planes buffers"));
        oc->scratch += xb + 3 * yb;
    }
    // buffers
    if (o.h_dtype == BPGB_DTYPE_F16) {
        e = cudaMalloc(&oc->rows, (size_t)num_pairs * oc->pitch16 * 2);
        oc->scratch += (uint64_t)num_pairs * oc->pitch16 * 2;
    }
    if (e == cudaSuccess) e = cudaMalloc(&oc->absmax, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&oc->coarse_vol, nc * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&oc->logits, nc * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&oc->feat, 2 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&oc->X, nc * oc->in_channels * 2);
    for (int k = 0; k < 3 && e == cudaSuccess; k++) e = cudaMalloc(&oc->Y[k], nc * 16 * 2);
    if (e == cudaSuccess) e = cudaMalloc(&oc->tile_list, oc->tiles * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&oc->tile_count, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(oc->tile_count, 0, sizeof(uint32_t));
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? set_error(BPGB_ERR_OUT_OF_MEMORY, "octree buffers")
                                                   : cuda_error(e, "octree buffers"));
    oc->scratch += nc * (4 + 4 + 2 * oc->in_channels + 3 * 32) + oc->tiles * 4 + 16;
    *out = oc;
    return BPGB_OK;
}

int bpgb_octree_reconstruct(bpgb_octree oc, const float *d_H, float *d_volume, void *stream) {
    clear_error();
    if (!oc || !d_H || !d_volume) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    oc->last = s;
    const void *rows = d_H;
    int st;
    const bool f16 = oc->h_dtype == BPGB_DTYPE_F16;
    if (f16) {
        st = bpgb_rows_absmax(d_H, oc->P, oc->T, oc->T, oc->absmax, s);
        if (st) return st;
        st = bpgb_rows_to_half(d_H, oc->P, oc->T, oc->T, 1.0f, oc->absmax, kHTarget,
                               BPGB_DTYPE_F16, oc->rows, oc->pitch16, s);
        if (st) return st;
        rows = oc->rows;
    }
    if ((st = bpgb_plan_execute(oc->coarse_plan, rows, oc->coarse_vol, s))) return st;
    if (oc->in_channels == 2)
        st = bpgb_cnn_features(oc->coarse_vol, oc->coarse, 1, oc->X, oc->feat, s);
    else
        st = bpgb_cnn_normalize(oc->coarse_vol, oc->coarse, 1, oc->X, s);
    if (st) return st;
    const void *in = oc->X;
    uint32_t xs = oc->in_channels;
    if (oc->tc) {
        // tcgen05 kernels on line-planes tensors
        if ((st = bpgb_cnn_lp_pack(oc->X, oc->in_channels, oc->in_channels, oc->coarse, 1, 0, oc->Xl, s)))
            return st;
        in = oc->Xl;
        for (size_t li = 0; li < oc->layers.size(); li++) {
            const Layer &L = oc->layers[li];
            const bool last = li + 1 == oc->layers.size();
            st = bpgb_cnn_tc_conv3d(in, L.cin, 0, oc->coarse, 1, oc->wtc[li],
                                    oc->master[li] + 27 * L.cin * L.cout, L.cout, L.relu ? 1 : 0,
                                    nullptr, last ? nullptr : oc->Yl[li], 0,
                                    last ? oc->logits : nullptr, s);
            if (st) return st;
            if (!last) in = oc->Yl[li];
        }
    }
    for (size_t li = 0; li < oc->layers.size() && !oc->tc; li++) {
        const Layer &L = oc->layers[li];
        const bool last = li + 1 == oc->layers.size();
        st = bpgb_cnn_conv3d(in, L.cin, xs, oc->coarse, 1, oc->wt[li], L.np, L.relu ? 1 : 0,
                             nullptr, 0, last ? nullptr : oc->Y[li], last ? oc->logits : nullptr,
                             s);
        if (st) return st;
        in = oc->Y[li];
        xs = 16;
    }
    if ((st = bpgb_upsample_trilinear(oc->coarse_vol, oc->coarse, d_volume, oc->fine, s))) return st;
    const uint32_t blocks[3] = {oc->coarse[0], oc->coarse[1], oc->coarse[2]};
    if ((st = bpgb_plan_select_tiles(oc->sparse_plan, oc->logits, blocks, kBlock, oc->logit_lo,
                                     oc->tile_list, oc->tile_count, s)))
        return st;
    if ((st = bpgb_plan_execute_tiles(oc->sparse_plan, rows, d_volume, oc->tile_list,
                                      oc->tile_count, oc->tiles, s)))
        return st;
    if (f16) {
        const uint64_t n = (uint64_t)oc->fine[0] * oc->fine[1] * oc->fine[2];
        if ((st = bpgb_volume_scale(d_volume, n, 1.0f, oc->absmax, kHTarget, s))) return st;
    }
    return BPGB_OK;
}

int bpgb_octree_reconstruct_host(bpgb_octree oc, const float *h_H, float *h_volume) {
    clear_error();
    if (!oc || !h_H || !h_volume) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    const size_t hb = (size_t)oc->P * oc->T * sizeof(float);
    const size_t vb = (size_t)oc->fine[0] * oc->fine[1] * oc->fine[2] * sizeof(float);
    if (!oc->io_H) {
        cudaError_t e = cudaMalloc(&oc->io_H, hb);
        if (e == cudaSuccess) e = cudaMalloc(&oc->io_vol, vb);
        if (e != cudaSuccess) {
            cudaFree(oc->io_H);
            cudaFree(oc->io_vol);
            oc->io_H = oc->io_vol = nullptr;
            return e == cudaErrorMemoryAllocation ? set_error(BPGB_ERR_OUT_OF_MEMORY, "octree I/O buffers")
                                                  : cuda_error(e, "octree I/O buffers");
        }
        oc->scratch += hb + vb;
    }
    BPGB_CUDA_TRY(cudaMemcpy(oc->io_H, h_H, hb, cudaMemcpyHostToDevice));
    int st = bpgb_octree_reconstruct(oc, oc->io_H, oc->io_vol, nullptr);
    if (st) return st;
    BPGB_CUDA_TRY(cudaMemcpy(h_volume, oc->io_vol, vb, cudaMemcpyDeviceToHost));
    uint64_t v = 0;
    return bpgb_plan_check(oc->sparse_plan, &v);
}

int bpgb_octree_selected(bpgb_octree oc, uint32_t *tiles) {
    clear_error();
    if (!oc || !tiles) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    BPGB_CUDA_TRY(cudaStreamSynchronize(oc->last));
    BPGB_CUDA_TRY(cudaMemcpy(tiles, oc->tile_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    uint64_t v = 0;
    return bpgb_plan_check(oc->sparse_plan, &v);
}

int bpgb_octree_get_info(bpgb_octree oc, bpgb_octree_info *info) {
    if (!oc || !info) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(info, 0, sizeof(*info));
    for (int k = 0; k < 3; k++) {
        info->fine[k] = oc->fine[k];
        info->coarse[k] = oc->coarse[k];
        info->tile[k] = oc->tile[k];
    }
    info->tiles = oc->tiles;
    info->in_channels = oc->in_channels;
    info->pair_splits = oc->pair_splits;
    info->h_dtype = oc->h_dtype;
    info->p_lo = oc->p_lo;
    info->scratch_bytes = oc->scratch;
    return BPGB_OK;
}

int bpgb_octree_destroy(bpgb_octree oc) {
    octree_free(oc);
    return BPGB_OK;
}

}  // extern "C"
