// Synthetic transient renderer and Poisson noise (see include/bpgb_synth.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "bpgb_internal.h"
#include "bpgb_synth.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Uniform in (0, 1) from (seed, index, draw).
inline double uniform(uint64_t seed, uint64_t index, uint64_t draw) {
    const uint64_t r = splitmix64(seed ^ splitmix64(index * 0x100000001B3ull + draw));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

double poisson_sample(double lam, uint64_t seed, uint64_t index) {
    if (!(lam > 0.0)) return 0.0;
    if (lam < 30.0) {
        const double L = std::exp(-lam);
        double p = 1.0;
        uint64_t k = 0;
        do {
            p *= uniform(seed, index, k);
            k++;
        } while (p > L && k < 1000);
        return (double)(k - 1);
    }
    const double u1 = uniform(seed, index, 0), u2 = uniform(seed, index, 1);
    const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    return std::max(0.0, std::floor(lam + std::sqrt(lam) * z + 0.5));
}

}  // namespace

extern "C" {

int bpgb_synth_render(const bpgb_pair *pairs, uint64_t num_pairs, uint32_t T, float t0,
                      float deltaT, const float *points, const float *albedo,
                      uint64_t num_points, float *out) {
    bpgb::clear_error();
    if ((num_pairs && (!pairs || !out)) || (num_points && (!points || !albedo)) || T == 0 ||
        !(deltaT > 0.0f))
        return bpgb::set_error(BPGB_ERR_INVALID_ARGUMENT, "bad render arguments");
    const double dT = deltaT;
#pragma omp parallel
    {
        std::vector<double> row(T);
#pragma omp for schedule(dynamic, 8)
        for (int64_t p = 0; p < (int64_t)num_pairs; p++) {
            std::fill(row.begin(), row.end(), 0.0);
            const bpgb_pair &pr = pairs[p];
            for (uint64_t i = 0; i < num_points; i++) {
                const float *q = points + 3 * i;
                double a2 = 0.0, b2 = 0.0;
                for (int k = 0; k < 3; k++) {
                    const double da = (double)pr.laser_point[k] - q[k];
                    const double db = (double)q[k] - pr.camera_point[k];
                    a2 += da * da;
                    b2 += db * db;
                }
                const double d = (double)pr.laser_wall + std::sqrt(a2) + std::sqrt(b2) +
                                 (double)pr.camera_wall;
                const double b = std::round((d - (double)t0) / dT);
                if (b < 0.0 || b >= (double)T || a2 <= 0.0 || b2 <= 0.0) continue;
                row[(uint32_t)b] += (double)albedo[i] / (a2 * b2);
            }
            float *o = out + (uint64_t)p * T;
            for (uint32_t t = 0; t < T; t++) o[t] = (float)row[t];
        }
    }
    return BPGB_OK;
}

int bpgb_synth_poisson(float *H, uint64_t n, float peak, uint64_t seed) {
    bpgb::clear_error();
    if (n && !H) return bpgb::set_error(BPGB_ERR_INVALID_ARGUMENT, "H is null");
    if (!(peak > 0.0f) || n == 0) return BPGB_OK;
    float mx = 0.0f;
#pragma omp parallel for reduction(max : mx)
    for (int64_t i = 0; i < (int64_t)n; i++) mx = std::max(mx, H[i]);
    if (!(mx > 0.0f)) return BPGB_OK;
    const double scale = (double)peak / (double)mx;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++)
        H[i] = (float)poisson_sample((double)H[i] * scale, seed, (uint64_t)i);
    return BPGB_OK;
}

}  // extern "C"
