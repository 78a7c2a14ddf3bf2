// Influence functions of the nonlocal model, shared by the pair assembly and
// the flux post-processing.
#pragma once

#include "common.cuh"

namespace nlgpu {

__device__ __forceinline__ double ipow(double x, int n) {   // power(T, integral) of metamath/functions/power.hpp:25-40
    double r = 1.0;
    while (n > 0) { if (n & 1) { r *= x; --n; } else { x *= x; n >>= 1; } }
    return r;
}

// Influence function without its normalisation (influence_functions_2d.hpp:39-148),
// over the powered distance of search_function.hpp:29-73 with the radii as
// inverse multipliers.
template<int INF>
__device__ __forceinline__ double shape(const Model& m, double dx, double dy) {
    const double z0 = dx * m.inv_r[0], z1 = dy * m.inv_r[1];
    double d;
    if (m.n == 2) d = z0 * z0 + z1 * z1;
    else if (m.n == 1) d = fabs(z0) + fabs(z1);
    else d = ipow(fabs(z0), m.n) + ipow(fabs(z1), m.n);
    if constexpr (INF == NLGPU_INFLUENCE_FAST_POLYNOMIAL) {
        return d < 1.0 ? 1.0 - d : 0.0;
    } else if constexpr (INF == NLGPU_INFLUENCE_CONSTANT) {
        return d <= 1.0 ? 1.0 : 0.0;
    } else {
        const bool integral = (m.p % m.n) == 0;
        const double dp = integral ? ipow(d, m.p / m.n) : pow(d, double(m.p) / double(m.n));
        if constexpr (INF == NLGPU_INFLUENCE_POLYNOMIAL) return d < 1.0 ? ipow(1.0 - dp, int(m.q)) : 0.0;
        else return exp(-m.q * dp);
    }
}

}  // namespace nlgpu
