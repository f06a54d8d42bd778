// Landing of FP64 sums into shared accumulators (the reverse product's
// scatter: point and cluster moments, face and node adjoints).
//
// By default a landing is one FP64 atomicAdd, whose order, and so whose
// rounding, varies from run to run.  With the option `deterministic` the
// library runs each scattering stage twice with its accumulators registered
// here:
//   pass 1: every landing raises its target's exponent E (the largest
//           ilogb of a value landed there) with an integer atomicMax;
//   pass 2: every landing adds its value as a 192-bit two's-complement
//           fixed-point number, 2^E at bit 126 (64 bits of headroom above the
//           largest value, values below 2^(E-126) truncated toward zero),
//           with three 64-bit integer atomicAdds and explicit carries.
// Integer addition is associative, so the final 192-bit sums, and the
// doubles converted from them (added to what the accumulators held), are the
// same whatever order the landings took.  A landing outside the registered
// arrays stays a plain atomicAdd.
//
// The kernels that land are templates on DET: their default instantiations
// compile to plain atomics, the DET ones read the state, which lives in
// constant memory, one copy per translation unit that lands (each defines a
// setter with IDW_LAND_SETTER); the host sets every copy on the launching
// stream before a pass and clears them after.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace idw {

constexpr int kLandArrays = 3;
constexpr int kLandNone = -2139062144;   // no landing: the int of four 0x80 bytes (the memset pattern)
constexpr int kLandNonFinite = 1 << 30;  // exponent of a target that received a NaN or an infinity

// Plain data (constant memory takes no initialiser): value-initialise on the host.
struct LandState {
    int pass;  // 0: plain atomics; 1: exponents; 2: fixed-point sums
    int nArr;
    double *base[kLandArrays];
    int64_t len[kLandArrays];
    int *expo[kLandArrays];               // per element
    unsigned long long *fix[kLandArrays];  // 3 per element
};

static __constant__ LandState c_land;

// 192-bit fixed-point add of v into w[0..2] (w[0] least significant), 2^E at
// bit 126.
__device__ __forceinline__ void land_fixed(unsigned long long *w, int E, double v) {
    if (v == 0.0 || E == kLandNone || E == kLandNonFinite) return;
    int e;
    const double m = frexp(fabs(v), &e);  // |v| = m 2^e, 0.5 <= m < 1
    const unsigned long long M = (unsigned long long)(m * 9007199254740992.0);  // m 2^53, exact
    // e <= E + 1 (pass 1 saw this value), so sh <= 74 and M << sh < 2^127
    const int sh = min(e - 53 + 126 - E, 74);
    unsigned long long u0 = 0, u1 = 0, u2 = 0;
    if (sh >= 64) {
        u1 = M << (sh - 64);
    } else if (sh > 0) {
        u0 = M << sh;
        u1 = M >> (64 - sh);
    } else if (sh > -64) {
        u0 = M >> (-sh);
    }
    if (v < 0.0) {  // two's complement over 192 bits
        u0 = ~u0 + 1ull;
        const unsigned long long c0 = u0 == 0ull ? 1ull : 0ull;
        u1 = ~u1 + c0;
        const unsigned long long c1 = (c0 && u1 == 0ull) ? 1ull : 0ull;
        u2 = ~u2 + c1;
    }
    const unsigned long long o0 = atomicAdd(&w[0], u0);
    const unsigned long long k0 = (o0 + u0 < o0) ? 1ull : 0ull;  // carry out of word 0
    const unsigned long long a1 = u1 + k0;
    const unsigned long long k1a = (a1 < u1) ? 1ull : 0ull;
    const unsigned long long o1 = atomicAdd(&w[1], a1);
    const unsigned long long k1 = ((o1 + a1 < o1) ? 1ull : 0ull) + k1a;  // carry out of word 1
    const unsigned long long a2 = u2 + k1;
    if (a2) atomicAdd(&w[2], a2);
}

// A landing of a deterministic kernel: the pass that is set, or an atomic
// for an address outside the registered arrays.
static __device__ __noinline__ void land_pass(double *d, double v) {
    for (int a = 0; a < c_land.nArr; ++a) {
        const int64_t t = d - c_land.base[a];
        if (t >= 0 && t < c_land.len[a]) {
            if (c_land.pass == 1) {
                if (v != 0.0) atomicMax(&c_land.expo[a][t], isfinite(v) ? ilogb(v) : kLandNonFinite);
            } else {
                land_fixed(c_land.fix[a] + 3 * t, c_land.expo[a][t], v);
            }
            return;
        }
    }
    atomicAdd(d, v);
}

// Adds v to *d.  DET = false (every kernel's default instantiation): one
// FP64 atomic, nothing else; DET = true (the instantiations launched for the
// option deterministic): the pass that is set.
template <bool DET>
__device__ __forceinline__ void land_add(double *d, double v) {
    if constexpr (DET) {
        if (c_land.pass != 0) {
            land_pass(d, v);
            return;
        }
    }
    atomicAdd(d, v);
}

}  // namespace idw

// A translation unit that lands defines its setter of c_land with this macro.
#define IDW_LAND_SETTER(name)                                                                         \
    cudaError_t name(const idw::LandState &s, cudaStream_t st) {                                      \
        return cudaMemcpyToSymbolAsync(idw::c_land, &s, sizeof(idw::LandState), 0, cudaMemcpyHostToDevice, st); \
    }
