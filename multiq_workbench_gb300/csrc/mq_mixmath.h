// Device helpers shared by the mixed-precision kernels (mq_mixed.cu, mq_tandem_mixed.cu): the
// Philox counter generator and its uniforms, the thermal-gas collision partner, double-float sums,
// 256-bit loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mqx {

// ---------------------------------------------------------------- Philox-4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11).
__device__ __forceinline__ uint4 philox(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return make_uint4(c0, c1, c2, c3);
}
__device__ __forceinline__ float unif(uint32_t x) { return (float)(x >> 8) * 0x1.0p-24f; }   // top 24 bits
__device__ __forceinline__ float unif16(uint32_t x16) { return (float)x16 * 0x1.0p-16f; }      // a 16-bit field
// sin / cos of a uniform angle 2 pi u - pi (u in [0, 1)): the hardware approximations are accurate to
// about 2^-21 on [-pi, pi], far below the Monte Carlo noise of the draws they serve, and a uniform
// angle shifted by pi is still uniform
__device__ __forceinline__ void angle_sincos(float u, float* s, float* c) { __sincosf(fmaf(u, 6.28318531f, -3.14159265f), s, c); }

// ---------------------------------------------------------------- thermal collision partner
// Null-collision sampling of hard-sphere collisions with a Maxwellian gas (gas velocity V with
// per-component spread s): the collision rate is n sigma E|v - V| and the partner of a collision
// has the density |v - V| f(V) / E|v - V|. The reference (world.rs:473-488) draws candidates at
// rate n sigma (|v| + 6 s), draws V from f and accepts with |v - V| / (|v| + 6 s). Here candidates
// come at rate n sigma (|v| + E|V|), E|V| = 2 sqrt(2/pi) s (the mean of the Maxwell speed
// distribution), and V from the proposal q(V) = f(V) (|v| + |V|) / (|v| + E|V|), accepted with
// |v - V| / (|v| + |V|) <= 1 (triangle inequality). The accepted rate density is
// n sigma (|v| + E|V|) q(V) |v - V| / (|v| + |V|) = n sigma f(V) |v - V|: the same collision process,
// exactly (a gas speed above 6 s, about 1e-7 of the draws, can exceed the 6 s bound; this bound
// holds for every draw), with a candidate rate 2 to 3.4 times smaller (ion speeds from 3 s down to
// 0.2 s). q is a two-part mixture: with probability |v| / (|v| + E|V|) the Maxwellian f itself
// (Box-Muller), else the speed-weighted Maxwellian |V| f(V) / E|V|, whose speed r has
// r^2 / 2 s^2 ~ Gamma(2, 1) = -ln(u1 u2) and whose direction is uniform. Uses from r: x, y (24-bit uniforms of the radii), z (two 16-bit angles or
// cos theta and an angle), w >> 16 (the mixture choice); w & 0xffff is left for the acceptance.
constexpr float kMeanSpeed = 1.59576912f;   // E|V| / s = 2 sqrt(2 / pi)

__device__ __forceinline__ void thermal_partner(uint4 r, float s, float vm, const float v[3], float gv[3], float& vm_sum) {
    const float ev = kMeanSpeed * s;
    const float ua = fmaxf(unif(r.x), 0x1.0p-25f), ub = fmaxf(unif(r.y), 0x1.0p-25f);
    float sa, ca;
    angle_sincos(unif16(r.z >> 16), &sa, &ca);
    float V[3], Vm;
    if (unif16(r.w >> 16) * (vm + ev) < vm) {          // V from f
        const float g1 = sqrtf(-2.0f * __logf(ua)), g2 = sqrtf(-2.0f * __logf(ub));
        float sb, cb;
        angle_sincos(unif16(r.z & 0xffffu), &sb, &cb);
        V[0] = s * (g1 * ca); V[1] = s * (g1 * sa); V[2] = s * (g2 * cb);
        Vm = s * sqrtf(fmaf(g1, g1, (g2 * cb) * (g2 * cb)));
    } else {                                            // V from |V| f(V) / E|V|
        Vm = s * sqrtf(-2.0f * __logf(ua * ub));
        const float ct = 2.0f * unif16(r.z & 0xffffu) - 1.0f;
        const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        V[0] = Vm * (st * ca); V[1] = Vm * (st * sa); V[2] = Vm * ct;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) gv[d] = v[d] - V[d];
    vm_sum = vm + Vm;
}

// ---------------------------------------------------------------- double-float helpers
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// 32 bytes from a 32-byte aligned address (ld.global.nc.v8.f32, sm_100 and later): two float4
__device__ __forceinline__ void ld256(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w) : "l"(p));
}

__device__ __forceinline__ int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace mqx
