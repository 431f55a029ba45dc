// Batched mixed-precision ion-trajectory engine for sm_103a.
//
// Same physics as the FP64 integrator (simulation/mqviz/src/world.rs:498-536 with chsim's
// switches, simulation/chsim/src/channel.metal:70-124), re-shaped for throughput:
//   * persistent workers: each lane pulls ions from a device work queue (one warp-
//     aggregated atomic per refill) and advances its ion until it finishes or has done
//     `chunk` steps; survivors are appended to the next launch's list by warp-ballot
//     compaction, so every launch starts with dense warps (chsim tc_filter + tc_tail,
//     channel_tiled.metal:341-482);
//   * positions in grid units and velocities in cells per step, each an FP32 double-float
//     (compensated two-sum accumulator); field nodes, interpolation and collision
//     kinematics in FP32;
//   * fields as interleaved node records of 64 bytes (256-bit loads) or 48 bytes, by grid size;
//     the 8 corners of the ion's cell x {RF, DC, AC} held in registers and reloaded only when
//     the ion changes cell (the cached conductor bits of the corners give the nearest-node
//     crash test), with an optional L1 prefetch of the cell the ion is heading for;
//   * RF / AC phase as exact 64-bit fixed-point turn accumulators (phase = offset +
//     step * f * dt mod 1), evaluated with an FP32 quarter-turn polynomial;
//   * Philox-4x32-10 counter RNG keyed by the ion's 64-bit key, counter = step (thermal candidates
//     and collisions) or 4-step window (legacy collisions: two blocks per window); thermal
//     candidates drawn against the majorant |v| + E|V| (mqx::thermal_partner), which samples the
//     reference's collision process with 2 to 3.4 times fewer candidates than its |v| + 6 s_gas;
//   * device injection with the FP64 injection's draws and FP32 transforms (k_inject_mixed).
#include "mq_mixed.h"
#include "mq_check.h"
#include "mq_mixmath.h"

#include <cstring>
#include <vector>

namespace mqmix {
namespace {

using mqd::DevGrid;
using mqd::DevIons;
using namespace mqx;

constexpr unsigned FULL = 0xffffffffu;

struct Ctrs {                       // device counters (40 B)
    uint32_t head;                  // work-queue head of the current launch
    uint32_t count[2];              // live-list lengths (ping-pong)
    uint32_t pad;
    unsigned long long steps;       // executed ion-steps
    unsigned long long cell_loads;  // cell-cache fills (8 node records each)
    unsigned long long queued;      // ions queued over the call's launches
};

// ---------------------------------------------------------------- FP32 turn-based sine
// sin / cos Taylor polynomials on [-pi/4, pi/4] (coefficients (-1)^k/(2k+1)!, (-1)^k/(2k)!)
__device__ __forceinline__ float sinp(float x) {
    float z = x * x;
    float p = fmaf(z, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    p = fmaf(z, p, 0x1.111112p-7f);
    p = fmaf(z, p, -0x1.555556p-3f);
    return fmaf(x * z, p, x);
}
__device__ __forceinline__ float cosp(float x) {
    float z = x * x;
    float p = fmaf(z, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    p = fmaf(z, p, -0x1.6c16c2p-10f);
    p = fmaf(z, p, 0x1.555556p-5f);
    return fmaf(z * z, p, fmaf(z, -0.5f, 1.0f));
}
// sin and cos of 2 pi P / 2^64 for a 64-bit fixed-point phase in turns
__device__ __forceinline__ void turn_sincos(uint64_t P, float& so, float& co) {
    int64_t r = (int64_t)(P << 2);                      // remainder of 4*phase in [-1/2, 1/2) quarter turns
    uint32_t q = (uint32_t)(P >> 62) + (r < 0 ? 1u : 0u);
    float x = (float)(int32_t)(r >> 32) * 0x1.921fb6p-32f;   // (pi/2) * 2^-32
    float s = sinp(x), c = cosp(x);
    float vs = (q & 1u) ? c : s, vc = (q & 1u) ? -s : c;
    so = (q & 2u) ? -vs : vs;
    co = (q & 2u) ? -vc : vc;
}
// one step of the drive: rotate (s, c) by the per-step angle (cw, sw)
__device__ __forceinline__ void rotate(float& s, float& c, float cw, float sw) {
    const float s2 = fmaf(s, cw, c * sw);
    c = fmaf(c, cw, -(s * sw));
    s = s2;
}

// ---------------------------------------------------------------- cell cache
// Interleaved node records: node q occupies float4 [Sq] = {RF.xyz, conductor mask},
// [Sq+1] = {combined DC.xyz, conductor bits of the cell based at q}, [Sq+2] = {AC.xyz, 0}, with
// a record stride S of 3 float4 (48 B) or 4 (64 B, the last float4 spare), so the 8 corners of a
// cell are 4 runs of 2 records. Wide records are 64-byte aligned and read with two 256-bit loads
// each (16 loads a reload instead of 24): faster where the cell reloads hit L2 (about 5% on the
// 0.100 mm channel), slower on fine grids whose gathers reach HBM and pay for the 33% larger
// footprint (0.050 mm: 10.7 against 17.3 G ion-steps/s).
struct Cell {
    float R[3][8], D[3][8], A[3][8];   // corner values per field and component, corner q = a + 2b + 4c
    int32_t ci, cj, ck;
    float fci, fcj, fck;                // the same cell as floats (no int -> float conversion per step)
    uint32_t mask;                      // conductor bit per corner
};

// record offsets are 32-bit (the host refuses grids with S x nodes >= 2^32): less address arithmetic
// in the divergent reload path (measured about 1% on the sweep)
__device__ __forceinline__ uint32_t node_of(const MixBatch& B, int32_t ci, int32_t cj, int32_t ck) {
    return (uint32_t)ci + (uint32_t)B.nx * ((uint32_t)cj + (uint32_t)B.ny * (uint32_t)ck);
}

// the same without allocating the lines in L1 (they are fetched from L2 into registers)
__device__ __forceinline__ void ld256_na(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.L1::no_allocate.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w) : "l"(p));
}

// NEAREST (the reference's legacy field mode: the field of the cell's lowest corner, t = 0) reads
// only that corner's record, which also holds the cell's conductor bits: one record per fill.
template <bool WIDE, bool NEAREST>
__device__ __forceinline__ void load_cell(const float4* __restrict__ nodes, const MixBatch& B, int32_t ci, int32_t cj,
                                          int32_t ck, Cell& c) {
    constexpr uint32_t S = WIDE ? 4u : 3u;
    const uint32_t sy = (uint32_t)B.nx, sz = (uint32_t)B.nx * (uint32_t)B.ny;
    const uint32_t base = node_of(B, ci, cj, ck);
    uint32_t m = 0;
#pragma unroll
    for (int q = 0; q < (NEAREST ? 1 : 8); ++q) {
        uint32_t o = S * (base + (uint32_t)(q & 1) + ((q & 2) ? sy : 0u) + ((q & 4) ? sz : 0u));
        o = (uint32_t)MQ_CHK_SPAN(o, S, S * (size_t)sz * (size_t)B.nz, MQ_SITE_MIX_CELL);
        float4 r, d, a;
        if (WIDE && !NEAREST) {
            // 64-byte records: both loads are 32-byte aligned. Wide records serve the grids whose
            // fills hit L2; left out of L1 they do not evict the lines the narrow-record grids
            // depend on either way (5% on the sweep; the fine grids' 48-byte fills lose 3x
            // without L1, so they keep it)
            float4 spare;
            ld256_na(nodes + o, r, d);
            ld256_na(nodes + o + 2, a, spare);
        } else if (WIDE) {
            float4 spare;
            ld256(nodes + o, r, d);
            ld256(nodes + o + 2, a, spare);
        } else {
            r = __ldg(nodes + o); d = __ldg(nodes + o + 1); a = __ldg(nodes + o + 2);
        }
        c.R[0][q] = r.x; c.R[1][q] = r.y; c.R[2][q] = r.z;
        c.D[0][q] = d.x; c.D[1][q] = d.y; c.D[2][q] = d.z;
        c.A[0][q] = a.x; c.A[1][q] = a.y; c.A[2][q] = a.z;
        if (q == 0) m = __float_as_uint(d.w);   // conductor bits of the cell's corners
    }
    c.ci = ci; c.cj = cj; c.ck = ck; c.mask = m;
    c.fci = (float)ci; c.fcj = (float)cj; c.fck = (float)ck;
}

// pull the 4 corner runs of a cell into L1 ahead of use
template <bool WIDE>
__device__ __forceinline__ void prefetch_cell(const float4* nodes, const MixBatch& B, int32_t ci, int32_t cj, int32_t ck) {
    const uint32_t sy = (uint32_t)B.nx, sz = (uint32_t)B.nx * (uint32_t)B.ny;
    const uint32_t base = node_of(B, ci, cj, ck);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float4* p = nodes + (WIDE ? 4 : 3) * (base + ((r & 1) ? sy : 0) + ((r & 2) ? sz : 0));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(p + (WIDE ? 7 : 5)));
    }
}

// E = a_rf RF(t) + DC(t) + a_ac AC(t): corner values combined first, then one trilinear pass
__device__ __forceinline__ float field_comp(const float R[8], const float D[8], const float A[8], float a_rf, float a_ac,
                                            float tx, float ty, float tz) {
    float F[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) F[q] = fmaf(a_rf, R[q], fmaf(a_ac, A[q], D[q]));
    const float c00 = fmaf(tx, F[1] - F[0], F[0]), c10 = fmaf(tx, F[3] - F[2], F[2]);
    const float c01 = fmaf(tx, F[5] - F[4], F[4]), c11 = fmaf(tx, F[7] - F[6], F[6]);
    const float c0 = fmaf(ty, c10 - c00, c00), c1 = fmaf(ty, c11 - c01, c01);
    return fmaf(tz, c1 - c0, c0);
}

// (xh + xl) - (th + tl) for a double-float position and threshold, as the sign-exact difference of
// two double-floats: xh - th is exact wherever the two are within a factor of 2 of each other (which
// covers every position close enough to the threshold for the low parts to matter), so the sign of
// the result is the sign of the unrounded difference there
__device__ __forceinline__ float df_diff(float xh, float xl, float th, float tl) {
    return __fadd_rn(__fsub_rn(xh, th), __fsub_rn(xl, tl));
}

// ---------------------------------------------------------------- the persistent worker
template <bool LEGACY, bool PREFETCH, bool WIDE, bool NEAREST>
__global__ void __launch_bounds__(128, 3)
k_mixed(const float4* __restrict__ nodes, MixBatch B, const MixJob* __restrict__ jobs, DevIons io,
        const uint32_t* __restrict__ list_in, uint32_t* __restrict__ list_out, Ctrs* ctr, int in_slot, uint32_t chunk,
        float* __restrict__ keep, const uint64_t* __restrict__ kph, uint32_t n_all) {
    // keep: the working state of every ion of the call in grid units, double-float position and
    // velocity (12 floats per ion, structure of arrays over n_all), filled from the FP64 states by
    // k_init_list and written back to them by k_unstage, so this kernel does no FP64 arithmetic;
    // kph: the RF / AC phase offsets as 64-bit fixed-point turns (two arrays of n_all)
    // The job constants only the collision branches read are staged per lane in shared memory at
    // refill, so those divergent branches do not wait on a global load (1.5% on the sweep, 5% on the
    // legacy-collision scan, against re-reading the job record there).
    __shared__ float sj_sgas[128], sj_mr[128], sj_floor[128], sj_mfp[128];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t count = ctr->count[in_slot];
    if (count == 0) return;
    uint32_t* count_out = &ctr->count[in_slot ^ 1];

    bool have = false, drained = false;
    uint32_t id = 0, jid = 0, n = 0, done = 0, ncoll = 0;
    int32_t leg = 0;
    float xh[3], xl[3], uh[3], ul[3];
    uint64_t Prf = 0, Pac = 0, Wac = 0;
    const uint64_t Wrf = ((uint64_t)B.w_rf_hi << 32) | B.w_rf_lo;
    // drive sines advanced by rotation each step and re-evaluated exactly from the
    // fixed-point phases every 4 loop iterations (warp-uniform), so rounding cannot build up
    float srf = 0.f, crf = 1.f, sac = 0.f, cac = 1.f, cw_ac = 1.f, sw_ac = 0.f;
    float kick = 0.f, v_ac = 0.f, cand_a = 0.f, cand_b = 0.f;
    uint32_t k0 = 0, k1 = 0;
    // per-step candidate uniforms: Philox block n>>2 (rc) and the next block (rn); rn is
    // refreshed for every lane on a warp-uniform schedule (every 4 loop iterations), so the
    // 10-round generator runs with all lanes active instead of once per lane-boundary
    uint4 rc = make_uint4(0, 0, 0, 0), rn = make_uint4(0, 0, 0, 0);
    uint32_t iter = 0;
    uint32_t loads = 0;                 // cell-cache fills of this lane
    Cell c;
    unsigned long long steps_total = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) { xh[d] = xl[d] = uh[d] = ul[d] = 0.f; }
    c.ci = c.cj = c.ck = -1; c.mask = 0;
    c.fci = c.fcj = c.fck = __int_as_float(0x7fc00000);   // NaN: differs from every floored position

    // Queue traffic is warp-synchronous and happens once every 4 iterations: survivors that ended in
    // the last 4 iterations are appended to the next launch's list, then lanes without an ion are
    // refilled (a lane that finished waits at most 3 iterations; 1.8% on the sweep and 3% on the
    // legacy scan against ballots every iteration).
    bool append = false;
    for (;;) {
      if ((iter & 3u) == 0u) {
        // ---- warp-ballot compaction of survivors into the next launch's list
        const unsigned am = __ballot_sync(FULL, append);
        if (am) {
            const int leader = __ffs(am) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(count_out, (uint32_t)__popc(am));
            base = __shfl_sync(FULL, base, leader);
            if (append) list_out[MQ_CHK(base + __popc(am & ((1u << lane) - 1u)), n_all, MQ_SITE_MIX_LIST_OUT)] = id;
        }
        append = false;
        // ---- refill: one warp-aggregated atomic hands out queue slots to lanes without an ion
        const unsigned need = __ballot_sync(FULL, !have && !drained);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(&ctr->head, (uint32_t)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (!have && !drained) {
                const uint32_t slot = base + __popc(need & ((1u << lane) - 1u));
                if (slot < count) {
                    id = (uint32_t)MQ_CHK(__ldg(list_in + slot), n_all, MQ_SITE_MIX_ION);
                    jid = io.jid[id];
                    const MixJob J = jobs[jid];
                    sj_sgas[threadIdx.x] = J.s_gas;
                    sj_mr[threadIdx.x] = J.mr;
                    sj_floor[threadIdx.x] = J.floor_v;
                    sj_mfp[threadIdx.x] = J.mfp_mean;
                    kick = J.kick; v_ac = J.use_ac ? J.v_ac : 0.0f; cand_a = J.cand_a; cand_b = J.cand_b;
                    Wac = ((uint64_t)J.w_ac_hi << 32) | J.w_ac_lo;
                    cw_ac = J.cw_ac; sw_ac = J.sw_ac;
                    n = io.steps[id]; ncoll = io.ncoll[id]; leg = io.leg[id];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        xh[d] = keep[(size_t)(0 + d) * n_all + id]; xl[d] = keep[(size_t)(3 + d) * n_all + id];
                        uh[d] = keep[(size_t)(6 + d) * n_all + id]; ul[d] = keep[(size_t)(9 + d) * n_all + id];
                    }
                    // phase = offset + n * w (mod 1) in 64-bit fixed point
                    const uint64_t orf = kph[id], oac = kph[(size_t)n_all + id];
                    Prf = orf + (uint64_t)n * Wrf;
                    Pac = oac + (uint64_t)n * Wac;
                    // drive state as an uninterrupted run has it: exact at the last step that is
                    // a multiple of 4, then rotated forward (so re-queued ions continue bitwise).
                    // An ion at a multiple of 4 steps (every fresh ion) first steps on a re-sync
                    // iteration, which sets its drive exactly and draws its next Philox block, so
                    // neither is done here for it
                    const uint32_t r4 = n & 3u;
                    if (r4) {
                        turn_sincos(Prf - (uint64_t)r4 * Wrf, srf, crf);
                        turn_sincos(Pac - (uint64_t)r4 * Wac, sac, cac);
                        for (uint32_t q = 0; q < r4; ++q) { rotate(srf, crf, B.cw_rf, B.sw_rf); rotate(sac, cac, cw_ac, sw_ac); }
                    }
                    const uint64_t key = io.rng[id];
                    k0 = (uint32_t)key; k1 = (uint32_t)(key >> 32);
                    if (!LEGACY) {
                        rc = philox(k0, k1, n >> 2, 0u, 0u, 0u);
                        if (r4) rn = philox(k0, k1, (n >> 2) + 1u, 0u, 0u, 0u);
                    } else if (r4) {   // the legacy collision words of the current 4-step window
                        rc = philox(k0, k1, n >> 2, 2u, 0u, 0u);
                        rn = philox(k0, k1, n >> 2, 3u, 0u, 0u);
                    }
                    load_cell<WIDE, NEAREST>(nodes, B, clampi(__float2int_rd(xh[0]), 0, B.nx - 2), clampi(__float2int_rd(xh[1]), 0, B.ny - 2),
                              clampi(__float2int_rd(xh[2]), 0, B.nz - 2), c);
                    ++loads;
                    done = 0;
                    have = true;
                } else {
                    drained = true;
                }
            }
        }
        if (!__any_sync(FULL, have)) break;
      }

        // A lane steps its ion only when the ion's step count is congruent to the warp's
        // iteration counter mod 4 (a freshly loaded ion waits at most 3 iterations).  Every
        // warp-uniform event below (Philox refresh and exact drive re-sync, each 4 iterations)
        // then falls on the same steps of every ion, whatever the scheduling, so per-ion
        // results are reproducible bit for bit.
        const bool act = have && (((iter ^ n) & 3u) == 0u);
        if (!LEGACY && (iter & 3u) == 0u && act) rn = philox(k0, k1, (n >> 2) + 1u, 0u, 0u, 0u);
        // legacy collisions draw from two Philox blocks per 4-step window, computed here with every
        // lane of the warp active (7% on the legacy scan against one block per collision inside
        // the divergent collision branch); a collision at window step q takes words 2q and 2q + 1
        if (LEGACY && (iter & 3u) == 0u && act) {
            rc = philox(k0, k1, n >> 2, 2u, 0u, 0u);
            rn = philox(k0, k1, n >> 2, 3u, 0u, 0u);
        }
        if ((iter & 3u) == 0u && act) { turn_sincos(Prf, srf, crf); turn_sincos(Pac, sac, cac); }
        ++iter;
        if (act) {
            // ---- field at the current position
            float tx = 0.f, ty = 0.f, tz = 0.f;
            if (!NEAREST) {
                tx = __fadd_rn(__fsub_rn(xh[0], c.fci), xl[0]);
                ty = __fadd_rn(__fsub_rn(xh[1], c.fcj), xl[1]);
                tz = __fadd_rn(__fsub_rn(xh[2], c.fck), xl[2]);
            }
            const float a_rf = B.v_rf * srf;
            const float a_ac = v_ac * sac;
            float E[3];
#pragma unroll
            for (int d = 0; d < 3; ++d)
                E[d] = NEAREST ? fmaf(a_rf, c.R[d][0], fmaf(a_ac, c.A[d][0], c.D[d][0]))   // = field_comp at t = 0
                               : field_comp(c.R[d], c.D[d], c.A[d], a_rf, a_ac, tx, ty, tz);
            // ---- kick (compensated) and drift (compensated)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                float inc = __fadd_rn(__fmul_rn(kick, E[d]), ul[d]);
                two_sum(uh[d], inc, uh[d], ul[d]);
                float s, e;
                fast_two_sum(xh[d], uh[d], s, e);
                e = __fadd_rn(e, __fadd_rn(xl[d], ul[d]));
                fast_two_sum(s, e, xh[d], xl[d]);
            }
            Prf += Wrf;
            Pac += Wac;
            rotate(srf, crf, B.cw_rf, B.sw_rf);
            rotate(sac, cac, cw_ac, sw_ac);
            const uint32_t nprev = n;
            n += 1;
            done += 1;
            // ---- collisions
            if (!LEGACY) {
                const float u0 = unif((nprev & 3) == 0 ? rc.x : (nprev & 3) == 1 ? rc.y : (nprev & 3) == 2 ? rc.z : rc.w);
                // candidate if u0 < cand_a |u| + cand_b = n sigma dt (|v| + E|V|), tested on squares
                // (no square root per step); see thermal_partner for why E|V| bounds the rate
                const float um2 = fmaf(uh[0], uh[0], fmaf(uh[1], uh[1], uh[2] * uh[2]));
                const float du = u0 - cand_b;
                if (du < 0.0f || du * du < cand_a * cand_a * um2) {
                    const float um = sqrtf(um2);
                    const float s_gas = sj_sgas[threadIdx.x], mr = sj_mr[threadIdx.x];
                    // two Philox blocks per candidate, drawn side by side: the first for the gas
                    // partner and the acceptance, the second for the scattering direction
                    const uint4 r0 = philox(k0, k1, nprev, 1u, 0u, 0u);
                    const uint4 r1 = philox(k0, k1, nprev, 2u, 0u, 0u);
                    const float u2v = B.u2v_f;
                    float v[3] = {uh[0] * u2v, uh[1] * u2v, uh[2] * u2v};
                    float gv[3], vm_sum;
                    thermal_partner(r0, s_gas, um * u2v, v, gv, vm_sum);
                    const float gl = sqrtf(fmaf(gv[0], gv[0], fmaf(gv[1], gv[1], gv[2] * gv[2])));
                    if (unif16(r0.w & 0xffffu) * vm_sum < gl) {
                        const float cth = 2.0f * unif(r1.x) - 1.0f;
                        float sp, cp;
                        angle_sincos(unif(r1.y), &sp, &cp);
                        const float sn = sqrtf(fmaxf(0.0f, 1.0f - cth * cth));
                        const float nn[3] = {sn * cp, sn * sp, cth};
                        const float v2u = B.v2u_f;
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            float vn = fmaf(mr * gl, nn[d], fmaf(-mr, gv[d], v[d]));
                            uh[d] = vn * v2u; ul[d] = 0.0f;
                        }
                        ncoll += 1;
                    }
                }
                if ((n & 3) == 0) rc = rn;   // rn holds block n>>2: refreshed at most 3 iterations ago
            } else {
                // a collision is due every ~4 steps per ion, so some lane of the warp needs one on
                // almost every iteration: every lane computes it and keeps it only where it is due,
                // with selects instead of a divergent branch
                leg -= 1;
                const bool due = leg <= 0;
                {
                    const float mr = sj_mr[threadIdx.x], floor_v = sj_floor[threadIdx.x], mfp_mean = sj_mfp[threadIdx.x];
                    // two 32-bit words of this window step: cos(theta) from the top 24 bits of the
                    // first, the free path from the top 24 of the second, phi from their low bytes
                    const uint32_t q = nprev & 3u;
                    const uint32_t wa = q == 0 ? rc.x : q == 1 ? rc.z : q == 2 ? rn.x : rn.z;
                    const uint32_t wb = q == 0 ? rc.y : q == 1 ? rc.w : q == 2 ? rn.y : rn.w;
                    const float u2v = B.u2v_f;
                    float v[3] = {uh[0] * u2v, uh[1] * u2v, uh[2] * u2v};
                    const float vm = sqrtf(fmaf(v[0], v[0], fmaf(v[1], v[1], v[2] * v[2])));
                    const bool hit = due && vm > floor_v;
                    const float cth = 2.0f * unif(wa) - 1.0f;
                    float sp, cp;
                    angle_sincos(unif16(((wa & 0xffu) << 8) | (wb & 0xffu)), &sp, &cp);
                    const float sn = sqrtf(fmaxf(0.0f, 1.0f - cth * cth));
                    const float dd[3] = {sn * cp, sn * sp, cth};
                    const float v2u = B.v2u_f;
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const float vn = fmaf(mr * vm, dd[d], v[d] * (1.0f - mr));
                        v[d] = hit ? vn : v[d];
                        uh[d] = hit ? vn * v2u : uh[d];
                        ul[d] = hit ? 0.0f : ul[d];
                    }
                    ncoll += hit ? 1u : 0u;
                    const float mfp = -__logf(fmaxf(unif(wb), 1e-7f)) * mfp_mean;
                    const float vn = sqrtf(fmaf(v[0], v[0], fmaf(v[1], v[1], v[2] * v[2])));
                    // free path in steps with the hardware's approximate division (within 2 ulp; the
                    // floored count moves by one step in rare ties, a few ions in 10^5; 3.8% on the
                    // legacy scan against two IEEE divisions)
                    const float st = floorf(__fdividef(mfp, fmaxf(vn, 1e-3f) * B.dt_f));
                    const int32_t nl = st < 1.0f ? 1 : (st < 2147483520.0f ? (int32_t)st : 2147483647);
                    leg = due ? nl : leg;
                }
            }
            // ---- cell of the new position (refresh the cache before the conductor test), and
            //      an L1 prefetch of the cell one more step ahead
            // cell changes are found on floored floats; indices are formed only when one is seen
            const float ffi = floorf(xh[0]), ffj = floorf(xh[1]), ffk = floorf(xh[2]);
            if (ffi != c.fci || ffj != c.fcj || ffk != c.fck) {
                const int32_t ci = clampi(__float2int_rd(xh[0]), 0, B.nx - 2), cj = clampi(__float2int_rd(xh[1]), 0, B.ny - 2),
                              ck = clampi(__float2int_rd(xh[2]), 0, B.nz - 2);
                if (ci != c.ci || cj != c.cj || ck != c.ck) { load_cell<WIDE, NEAREST>(nodes, B, ci, cj, ck, c); ++loads; }
            }
            if (PREFETCH && !NEAREST) {
                const int32_t pi = clampi(__float2int_rd(xh[0] + uh[0]), 0, B.nx - 2);
                const int32_t pj = clampi(__float2int_rd(xh[1] + uh[1]), 0, B.ny - 2);
                const int32_t pk = clampi(__float2int_rd(xh[2] + uh[2]), 0, B.nz - 2);
                if (pi != c.ci || pj != c.cj || pk != c.ck) prefetch_cell<WIDE>(nodes, B, pi, pj, pk);
            }
            // ---- termination tests: exit, return, box, conductor, timeout
            // (the loss-surface planes - exit, return and the crash window - are crossed on the full
            // double-float position against the double-float thresholds; the box test is the
            // unclamped cell index leaving [0, n-2])
            // A plane more than one cell away cannot be crossed whatever the low parts hold, so the
            // exact test runs only within a cell of it; the crash window matters only in a cell with
            // a conductor corner (most cells have none).
            int32_t status = 0;
            if (xh[2] > B.z_exit_near && df_diff(xh[2], xl[2], B.z_exit_h, B.z_exit_l) > 0.0f) status = 3;
            else if (xh[2] < B.z_ret_near && df_diff(xh[2], xl[2], B.z_ret_h, B.z_ret_l) < 0.0f) status = 2;
            else if (ffi < 0.0f || ffj < 0.0f || ffk < 0.0f || ffi > B.lim_x - 1.0f || ffj > B.lim_y - 1.0f ||
                     ffk > B.lim_z - 1.0f)
                status = 4;
            else {
                if (c.mask != 0u && df_diff(xh[2], xl[2], B.cz0_h, B.cz0_l) > 0.0f &&
                    df_diff(xh[2], xl[2], B.cz1_h, B.cz1_l) < 0.0f) {
                    const float fx = __fadd_rn(__fsub_rn(xh[0], c.fci), xl[0]);
                    const float fy = __fadd_rn(__fsub_rn(xh[1], c.fcj), xl[1]);
                    const float fz = __fadd_rn(__fsub_rn(xh[2], c.fck), xl[2]);
                    const uint32_t q = (fx >= 0.5f ? 1u : 0u) | (fy >= 0.5f ? 2u : 0u) | (fz >= 0.5f ? 4u : 0u);
                    if ((c.mask >> q) & 1u) status = 1;
                }
                if (status == 0 && n >= B.max_steps) status = 5;
            }
            if (status != 0 || done >= chunk) {
                // ---- write back: counters to the ion states, position and velocity to the working
                //      state (k_unstage turns it into the FP64 state when the caller wants that)
                io.steps[id] = n; io.ncoll[id] = ncoll; io.leg[id] = leg; io.status[id] = status;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    keep[(size_t)(0 + d) * n_all + id] = xh[d]; keep[(size_t)(3 + d) * n_all + id] = xl[d];
                    keep[(size_t)(6 + d) * n_all + id] = uh[d]; keep[(size_t)(9 + d) * n_all + id] = ul[d];
                }
                steps_total += done;
                append = status == 0;
                have = false;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        steps_total += __shfl_down_sync(FULL, steps_total, o);
        loads += __shfl_down_sync(FULL, loads, o);
    }
    if (lane == 0 && steps_total) atomicAdd(&ctr->steps, steps_total);
    if (lane == 0 && loads) atomicAdd(&ctr->cell_loads, (unsigned long long)loads);
}

// interleave RF | combined DC | AC into node records of `stride` float4 (once per DC configuration
// and record width); the spare w of the DC record holds the conductor bits of the 8 corners of the
// cell whose lowest corner is this node (bit a + 2b + 4c), so a cell reload reads its crash mask in
// one word
__global__ void k_pack_nodes(const float4* __restrict__ rf, const float4* __restrict__ dc, const float4* __restrict__ ac,
                             float4* __restrict__ nodes, size_t n, int32_t nx, int32_t ny, int32_t nz, int stride) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    nodes[stride * q] = rf[q];
    if (stride == 4) nodes[4 * q + 3] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 d = dc[q];
    const size_t sy = (size_t)nx, sz = (size_t)nx * (size_t)ny;
    const int32_t i = (int32_t)(q % sy), j = (int32_t)((q / sy) % (size_t)ny), k = (int32_t)(q / sz);
    uint32_t m = 0;
    if (i < nx - 1 && j < ny - 1 && k < nz - 1)
        for (int c = 0; c < 8; ++c)
            m |= (rf[q + (size_t)(c & 1) + ((c & 2) ? sy : 0) + ((c & 4) ? sz : 0)].w > 0.5f ? 1u : 0u) << c;
    d.w = __uint_as_float(m);
    nodes[stride * q + 1] = d;
    nodes[stride * q + 2] = ac[q];
}

// ---------------------------------------------------------------- injection for the mixed engine
// The draws of mqp::inject_one (Ion::inject, world.rs:407-422, with chsim's launches,
// channel.rs:342-366): the same seed, the same xorshift stream in the same order, so the ion's
// generator state and its RF / AC phases are the FP64 injection's bit for bit; the transforms of
// the draws (sqrt, log, sin / cos) run in FP32, as the reference's GPU path consumes FP32 ion
// states (its injection runs on the host, channel.rs:342-366, and is narrowed to f32 for the
// device). Positions take their FP32 offset from the axis in FP64, so they keep the axis exactly.
// GB300's FP64 pipe makes the FP64 transforms (about 360 FP64 operations per ion) the whole cost
// of the FP64 kernel k_inject; here an ion costs a few dozen FP32 operations.
__device__ __forceinline__ uint64_t xs_raw(uint64_t* st) {   // xorshift64 step, world.rs:386-392
    uint64_t x = *st;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *st = x;
    return x;
}
// (x >> 11) / 2^53 as FP32: top 24 bits plus the next 29 scaled below them (within 1 ulp)
__device__ __forceinline__ float u53f(uint64_t x) {
    return fmaf((float)((uint32_t)(x >> 11) & 0x1FFFFFFFu), 0x1.0p-53f, (float)(uint32_t)(x >> 40) * 0x1.0p-24f);
}
__device__ __forceinline__ double u53d(uint64_t x) { return (double)(x >> 11) * 0x1.0p-53; }   // exact
// -ln u for u = (x >> 11) / 2^53 > 0, to FP32 accuracy also near u = 1, where 1 - u is formed
// exactly in integers and the logarithm taken as log1p(-(1 - u))
__device__ __forceinline__ float neg_log_u(uint64_t x) {
    const uint64_t k = x >> 11;
    if (k >= (1ull << 52)) return -log1pf(-(float)((1ull << 53) - k) * 0x1.0p-53f);
    return -logf(u53f(x));
}
// sqrt(-2 ln max(u, 1e-300)): the FP64 clamp lies below FP32's range; only u = 0 reaches it
__device__ __forceinline__ float gauss_radius(uint64_t x) {
    return (x >> 11) ? sqrtf(2.0f * neg_log_u(x)) : 37.1692219f;
}

__global__ void __launch_bounds__(128) k_inject_mixed(mqp::Batch b, mqd::JobTable jt, DevIons io, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t lo = 0, hi = jt.njobs;   // the job of ion i: last job with first <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jt.first[mid] <= i) lo = mid; else hi = mid;
    }
    const mqp::JobC& j = jt.jc[lo];
    uint64_t st = mqp::splitmix(jt.seed[lo] + ((uint64_t)i - jt.first[lo]) * 0x9E37ull) | 1ull;
    float ox, oy, v0, v1, v2;
    if (b.launch == 1) {               // legacy launch, channel.rs:350-355
        const float kin = 0.1f * (0.75f + 0.75f * u53f(xs_raw(&st))) * (float)j.zc;
        const float vin = sqrtf(2.0f * kin * ((float)mqp::QE / (float)j.m));
        const float ang = (-10.0f + 20.0f * u53f(xs_raw(&st))) * (3.14159265f / 180.0f);
        float sa, ca;
        sincosf(ang, &sa, &ca);
        ox = oy = 0.0f;
        v0 = v1 = 0.707f * vin * sa;
        v2 = vin * ca;
    } else {
        if (b.launch == 2) {           // Gaussian spot
            const float r0 = gauss_radius(xs_raw(&st));
            const float c0 = cospif(2.0f * u53f(xs_raw(&st)));
            const float r1 = gauss_radius(xs_raw(&st));
            const float c1 = cospif(2.0f * u53f(xs_raw(&st)));
            ox = (float)b.sigma * r0 * c0;
            oy = (float)b.sigma * r1 * c1;
        } else {                       // uniform disc
            const float r = (float)b.r_inject * sqrtf(u53f(xs_raw(&st)));
            float sn, cs;
            sincospif(2.0f * u53f(xs_raw(&st)), &sn, &cs);
            ox = r * cs;
            oy = r * sn;
        }
        const float s_ion = (float)j.s_ion;
        const float ra = gauss_radius(xs_raw(&st));
        const float ca = cospif(2.0f * u53f(xs_raw(&st)));
        const float rb = gauss_radius(xs_raw(&st));
        const float cb = cospif(2.0f * u53f(xs_raw(&st)));
        v0 = s_ion * ra * ca;
        v1 = s_ion * rb * cb;
        v2 = s_ion * gauss_radius(xs_raw(&st));
    }
    const double ph_ac = u53d(xs_raw(&st));
    const double prf = u53d(xs_raw(&st));
    const uint64_t xf = xs_raw(&st);
    // first free path -ln max(u, 1e-7) * mfp / 10 (channel.rs:365-366) as a step count; u < 1e-7
    // exactly when (x >> 11) <= 900719925
    const float nl = (xf >> 11) <= 900719925ull ? 16.1180957f : neg_log_u(xf);
    const float first = nl * (float)j.mfp_mean / 10.0f;
    const float vmag = sqrtf(fmaf(v0, v0, fmaf(v1, v1, v2 * v2)));
    const float s0 = floorf(first / vmag / (float)b.dt) + 1.0f;
    io.x[i] = b.a + (double)ox; io.y[i] = b.a + (double)oy; io.z[i] = b.z_inject;
    io.vx[i] = (double)v0; io.vy[i] = (double)v1; io.vz[i] = (double)v2;
    io.ph_rf[i] = b.rf_phase0 ? 0.0 : prf; io.ph_ac[i] = ph_ac;
    io.rng[i] = st | 1ull;
    io.leg[i] = s0 < 2147483520.0f ? (int32_t)s0 : 2147483647;
    io.steps[i] = 0; io.ncoll[i] = 0; io.status[i] = 0; io.jid[i] = lo;
}

// initial live list (ions with status 0, warp-ballot compaction) and their working state: the
// FP64 position / velocity in grid units as double-floats and the phase offsets as fixed-point
// turns, converted here with every lane of a warp busy instead of one lane at a time in k_mixed
__global__ void k_init_list(DevIons io, uint32_t n, uint32_t* list, Ctrs* ctr, MixBatch B, float* __restrict__ keep,
                            uint64_t* __restrict__ kph, uint8_t* __restrict__ staged) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n && io.status[i] == 0;
    if (i < n) staged[i] = live ? 1 : 0;
    if (live) {
        const double gx[3] = {io.x[i] * B.inv_h, io.y[i] * B.inv_h, io.z[i] * B.inv_h};
        const double gu[3] = {io.vx[i] * B.v2u, io.vy[i] * B.v2u, io.vz[i] * B.v2u};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float xh = (float)gx[d], uh = (float)gu[d];
            keep[(size_t)(0 + d) * n + i] = xh; keep[(size_t)(3 + d) * n + i] = (float)(gx[d] - (double)xh);
            keep[(size_t)(6 + d) * n + i] = uh; keep[(size_t)(9 + d) * n + i] = (float)(gu[d] - (double)uh);
        }
        kph[i] = (uint64_t)(io.ph_rf[i] * 0x1.0p63) << 1;
        kph[(size_t)n + i] = (uint64_t)(io.ph_ac[i] * 0x1.0p63) << 1;
    }
    const unsigned m = __ballot_sync(FULL, live);
    const uint32_t lane = threadIdx.x & 31;
    if (m) {
        const int leader = __ffs(m) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&ctr->count[0], (uint32_t)__popc(m));
        base = __shfl_sync(FULL, base, leader);
        if (live) list[base + __popc(m & ((1u << lane) - 1u))] = i;
    }
}

// FP64 position and velocity of every ion staged at the start of the call, from its working state
__global__ void k_unstage(DevIons io, uint32_t n, MixBatch B, const float* __restrict__ keep,
                          const uint8_t* __restrict__ staged) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !staged[i]) return;
    double* const xs[3] = {io.x, io.y, io.z};
    double* const vs[3] = {io.vx, io.vy, io.vz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        xs[d][i] = ((double)keep[(size_t)(0 + d) * n + i] + (double)keep[(size_t)(3 + d) * n + i]) * B.h;
        vs[d][i] = ((double)keep[(size_t)(6 + d) * n + i] + (double)keep[(size_t)(9 + d) * n + i]) * B.u2v;
    }
}

// ---------------------------------------------------------------- cell order of the live list
// Before a launch, the live list can be put in the Morton order of the ions' cells (a counting sort
// on the top bits of the 30-bit code), so the 32 lanes of a warp, which take consecutive queue
// slots, start in neighbouring cells and share cache lines in their cell gathers.  Order within a
// bin is the atomics' arrival order: per-ion results do not depend on the order.
// Bits 0..9 of v spread to every third bit (the "part 1 by 2" step of Morton encoding).
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v ^ (v << 16)) & 0xff0000ffu;
    v = (v ^ (v << 8)) & 0x0300f00fu;
    v = (v ^ (v << 4)) & 0x030c30c3u;
    v = (v ^ (v << 2)) & 0x09249249u;
    return v;
}

constexpr int kScanBlock = 1024;          // threads of the scan kernels
constexpr int kScanItems = 4;             // bins per scan thread
constexpr uint32_t kScanTile = kScanBlock * kScanItems;

// bin of every listed ion (cell Morton code >> shift) and the bins' counts; lanes of a warp with the
// same bin add to it with one atomic (ions cluster in few cells, e.g. right after injection)
__global__ void k_sort_keys(const uint32_t* __restrict__ list, const Ctrs* __restrict__ ctr, int slot,
                            const float* __restrict__ keep, uint32_t n_all, MixBatch B, uint32_t shift,
                            uint32_t* __restrict__ keys, uint32_t* __restrict__ bins) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ctr->count[slot]) return;
    const uint32_t id = list[t];
    const uint32_t ci = (uint32_t)clampi(__float2int_rd(keep[(size_t)0 * n_all + id]), 0, B.nx - 2);
    const uint32_t cj = (uint32_t)clampi(__float2int_rd(keep[(size_t)1 * n_all + id]), 0, B.ny - 2);
    const uint32_t ck = (uint32_t)clampi(__float2int_rd(keep[(size_t)2 * n_all + id]), 0, B.nz - 2);
    const uint32_t key = (spread10(ci) | (spread10(cj) << 1) | (spread10(ck) << 2)) >> shift;
    keys[t] = key;
    const unsigned peers = __match_any_sync(__activemask(), key);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) atomicAdd(bins + key, (uint32_t)__popc(peers));
}

// exclusive scan of a tile of kScanTile counts in place; the tile's total to sums[blockIdx.x]
__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(uint32_t* __restrict__ v, uint32_t n, uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_tot[kScanBlock / 32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t x[kScanItems], run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        x[k] = base + k < n ? v[base + k] : 0u;
        run += x[k];
    }
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        warp_tot[lane] = t;   // inclusive over warps
    }
    __syncthreads();
    uint32_t off = inc - run + (w ? warp_tot[w - 1] : 0u);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) v[base + k] = off;
        off += x[k];
    }
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = warp_tot[kScanBlock / 32 - 1];
}

// add the scanned tile totals to every tile
__global__ void k_scan_add(uint32_t* __restrict__ v, uint32_t n, const uint32_t* __restrict__ sums) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] += sums[i / kScanTile];
}

// every listed ion to the next free place of its bin (one atomic per bin per warp)
__global__ void k_sort_scatter(const uint32_t* __restrict__ list, const Ctrs* __restrict__ ctr, int slot,
                               const uint32_t* __restrict__ keys, uint32_t* __restrict__ bins, uint32_t* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ctr->count[slot]) return;
    const uint32_t key = keys[t], lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(__activemask(), key);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(bins + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    out[base + __popc(peers & ((1u << lane) - 1u))] = list[t];
}

// prepare launch: clear the queue head and the output count, and add the launch's queue length
__global__ void k_prep(Ctrs* ctr, int out_slot) {
    ctr->head = 0;
    ctr->count[out_slot] = 0;
    ctr->queued += ctr->count[out_slot ^ 1];
}

void split(double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

uint64_t fix64(double turns_per_step) {   // round(frac(w) * 2^64)
    double f = turns_per_step - floor(turns_per_step);
    long double s = (long double)f * 18446744073709551616.0L;
    long double r = floorl(s + 0.5L);
    if (r >= 18446744073709551616.0L) return 0;
    return (uint64_t)r;
}

}  // namespace

cudaError_t launch_inject(const mqp::Batch& b, mqd::JobTable jt, DevIons io, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_inject_mixed<<<(n + 127) / 128, 128, 0, st>>>(b, jt, io, n);
    return cudaGetLastError();
}

MixJob make_mix_job(const mqp::JobC& j, const mqp::Batch& b) {
    MixJob m;
    std::memset(&m, 0, sizeof(m));
    m.kick = (float)(j.qmdt * b.dt / b.h);
    m.v_ac = (float)j.v_ac;
    m.cand_a = (float)(j.nsd * b.h / b.dt);
    m.cand_b = (float)(j.nsd * 1.5957691216057308 * j.s_gas);   // n sigma dt E|V| (thermal_partner)
    m.s_gas = (float)j.s_gas;
    m.mr = (float)j.mr;
    m.floor_v = (float)j.floor_v;
    m.mfp_mean = (float)j.mfp_mean;
    uint64_t w = fix64(j.w_ac);
    m.w_ac_lo = (uint32_t)w;
    m.w_ac_hi = (uint32_t)(w >> 32);
    double s, c;
    mqp::sincos2pi(j.w_ac, &s, &c);
    m.cw_ac = (float)c;
    m.sw_ac = (float)s;
    m.use_ac = j.use_ac;
    return m;
}

MixBatch make_mix_batch(const mqp::Batch& b) {
    MixBatch m;
    std::memset(&m, 0, sizeof(m));
    m.h = b.h;
    m.inv_h = 1.0 / b.h;
    m.dt = b.dt;
    m.u2v = b.h / b.dt;
    m.v2u = b.dt / b.h;
    m.v_rf = (float)b.v_rf;
    m.dt_f = (float)b.dt;
    m.u2v_f = (float)m.u2v;
    m.v2u_f = (float)m.v2u;
    uint64_t w = fix64(b.w_rf);
    m.w_rf_lo = (uint32_t)w;
    m.w_rf_hi = (uint32_t)(w >> 32);
    double s, c;
    mqp::sincos2pi(b.w_rf, &s, &c);
    m.cw_rf = (float)c;
    m.sw_rf = (float)s;
    split(b.z_exit / b.h, m.z_exit_h, m.z_exit_l);
    split(b.z_return / b.h, m.z_ret_h, m.z_ret_l);
    split(b.crash_z0 / b.h, m.cz0_h, m.cz0_l);
    split(b.crash_z1 / b.h, m.cz1_h, m.cz1_l);
    m.z_exit_near = m.z_exit_h - 1.0f;
    m.z_ret_near = m.z_ret_h + 1.0f;
    m.lim_x = (float)(b.nx - 1);
    m.lim_y = (float)(b.ny - 1);
    m.lim_z = (float)(b.nz - 1);
    m.nx = b.nx; m.ny = b.ny; m.nz = b.nz;
    m.nearest = b.nearest;
    m.legacy_coll = b.legacy_coll;
    m.max_steps = b.max_steps;
    return m;
}

Tuning default_tuning(int device, size_t nodes) {
    Tuning t;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) { cudaGetLastError(); sms = 1; }
    t.sms = sms;
    // Resident ions per SM by the size of the node records: on grids far larger than L2 the
    // gathers of fewer ions in flight hit the caches more often than more warps hide latency
    // (measured on the channel at 0.050 / 0.0333 mm, 2.4 / 8.0 GB of 48-byte records: 15.7 / 11.4
    // G ion-steps/s at 1 block per SM against 15.0 / 7.1 at 2 and 10.6 / - at 3; the 0.100 mm grid,
    // 0.30 GB, is best at 3). Wide records only in the first class: they win where the reloads hit
    // L2 and lose where they reach HBM.
    const double rec = 48.0 * (double)nodes;
    t.blocks_per_sm = rec < 1.0e9 ? 3 : 1;
    t.wide = rec < 1.0e9 ? 1 : 0;
    return t;
}

void release(Scratch& s) {
    if (s.graph) cudaGraphExecDestroy(s.graph);
    for (void* p : {s.lists, s.ctrs, s.params, s.jobs, s.nodes, s.keep, s.sort}) if (p) cudaFree(p);
    for (auto& e : s.ev) if (e) cudaEventDestroy(e);
    s = Scratch();
}

// the stepping kernel for the batch's physics and the tuning (the nearest-node field mode reads one
// record per fill, so the L1 prefetch of the next cell does not apply to it)
typedef decltype(&k_mixed<true, true, true, false>) Kernel;
static Kernel pick_kernel(const Tuning& t, const MixBatch& mb) {
    if (mb.nearest) {
        if (mb.legacy_coll) return t.wide ? k_mixed<true, false, true, true> : k_mixed<true, false, false, true>;
        return t.wide ? k_mixed<false, false, true, true> : k_mixed<false, false, false, true>;
    }
    if (mb.legacy_coll) {
        if (t.wide) return t.prefetch ? k_mixed<true, true, true, false> : k_mixed<true, false, true, false>;
        return t.prefetch ? k_mixed<true, true, false, false> : k_mixed<true, false, false, false>;
    }
    if (t.wide) return t.prefetch ? k_mixed<false, true, true, false> : k_mixed<false, false, true, false>;
    return t.prefetch ? k_mixed<false, true, false, false> : k_mixed<false, false, false, false>;
}

// bins of the cell sort: the top min(22, 3 b) bits of the Morton code, b the bits of the largest
// cell index (nbins <= 2^22, so the tile totals fit one scan tile)
struct SortPlan {
    uint32_t nbins, tiles, shift;
};
static SortPlan sort_plan(const MixBatch& mb, uint32_t n) {
    (void)n;
    int32_t mx = mb.nx > mb.ny ? mb.nx : mb.ny;
    mx = mx > mb.nz ? mx : mb.nz;
    uint32_t bits = 1;
    while ((1u << bits) < (uint32_t)(mx - 1)) ++bits;   // cell indices 0 .. mx - 2
    const uint32_t code = 3 * bits, kb = code < 22 ? code : 22;
    SortPlan p;
    p.nbins = 1u << kb;
    p.tiles = (p.nbins + kScanTile - 1) / kScanTile;
    p.shift = code - kb;
    return p;
}
static size_t sort_bytes(const MixBatch& mb, uint32_t n) {
    const SortPlan p = sort_plan(mb, n);
    return sizeof(uint32_t) * ((size_t)p.nbins + p.tiles + 1 + 2 * (size_t)n);
}

static cudaError_t enqueue_launches(const Scratch& s, const Tuning& t, int blocks_per_sm, const MixBatch& mb, DevIons io,
                                    uint32_t n, uint32_t launches, uint32_t chunk, uint32_t last_chunk, cudaStream_t st,
                                    uint32_t* kernels) {
    uint32_t* lists = static_cast<uint32_t*>(s.lists);
    Ctrs* ctr = static_cast<Ctrs*>(s.ctrs);
    const MixJob* jobs = static_cast<const MixJob*>(s.jobs);
    const float4* nodes = static_cast<const float4*>(s.nodes);
    uint64_t* kph = static_cast<uint64_t*>(s.keep);
    float* keep = reinterpret_cast<float*>(kph + (size_t)2 * n);
    const int grid = t.sms * blocks_per_sm;
    const SortPlan sp = sort_plan(mb, n);
    uint32_t* bins = static_cast<uint32_t*>(s.sort);
    uint32_t* sums = bins + sp.nbins;
    uint32_t* keys = sums + sp.tiles + 1;
    uint32_t* sorted = keys + n;
    for (uint32_t L = 0; L < launches; ++L) {
        const int in = (int)(L & 1);
        k_prep<<<1, 1, 0, st>>>(ctr, in ^ 1);
        const uint32_t ch = (L + 1 == launches) ? last_chunk : chunk;
        const uint32_t* li = lists + (size_t)in * n;
        uint32_t* lo = lists + (size_t)(in ^ 1) * n;
        if (t.sort_cells) {   // this launch's list in the cells' Morton order
            cudaMemsetAsync(bins, 0, (size_t)sp.nbins * sizeof(uint32_t), st);
            const unsigned gi = (n + 255) / 256;
            k_sort_keys<<<gi, 256, 0, st>>>(li, ctr, in, keep, n, mb, sp.shift, keys, bins);
            k_scan_tiles<<<sp.tiles, kScanBlock, 0, st>>>(bins, sp.nbins, sums);
            k_scan_tiles<<<1, kScanBlock, 0, st>>>(sums, sp.tiles, sums + sp.tiles);   // tiles <= kScanTile
            k_scan_add<<<(sp.nbins + 255) / 256, 256, 0, st>>>(bins, sp.nbins, sums);
            k_sort_scatter<<<gi, 256, 0, st>>>(li, ctr, in, keys, bins, sorted);
            li = sorted;
            *kernels += 5;
        }
        const Kernel kern = pick_kernel(t, mb);
        kern<<<grid, t.tpb, 0, st>>>(nodes, mb, jobs, io, li, lo, ctr, in, ch, keep, kph, n);
        *kernels += 2;
    }
    return cudaGetLastError();
}

cudaError_t pack_nodes(Scratch& s, DevGrid g, uint64_t grid_gen, int wide, cudaStream_t st, uint32_t* kernels) {
    const int stride = wide ? 4 : 3;
    if (s.nodes && s.nodes_gen == grid_gen && s.nodes_stride == stride) return cudaSuccess;
    cudaError_t e;
    const size_t n = (size_t)g.nx * g.ny * g.nz;
    const size_t bytes = (size_t)stride * n * sizeof(float4);
    if (s.nodes_cap < bytes) {
        if (s.nodes) cudaFree(s.nodes);
        s.nodes = nullptr; s.nodes_cap = 0;
        if ((e = cudaMalloc(&s.nodes, bytes)) != cudaSuccess) return e;
        s.nodes_cap = bytes;
    }
    k_pack_nodes<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g.rf, g.dc, g.ac, static_cast<float4*>(s.nodes), n, g.nx, g.ny, g.nz,
                                                              stride);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    *kernels += 1;
    s.nodes_gen = grid_gen;
    s.nodes_stride = stride;
    return cudaSuccess;
}

cudaError_t run(Scratch& s, const Tuning& t, DevGrid g, uint64_t grid_gen, const mqp::Batch& b, const MixJob* jobs,
                size_t njobs, DevIons io, uint32_t n, uint32_t max_more, int write_states, cudaStream_t st, RunInfo* info) {
    cudaError_t e;
    *info = RunInfo();
    if (n == 0) return cudaSuccess;
    if (t.tpb != 128) return cudaErrorInvalidValue;   // the kernel is compiled for 128-thread blocks
    if ((e = pack_nodes(s, g, grid_gen, t.wide, st, &info->kernel_launches)) != cudaSuccess) return e;
    const size_t list_bytes = (size_t)2 * n * sizeof(uint32_t);
    if (s.list_cap < list_bytes) {
        if (s.lists) cudaFree(s.lists);
        s.lists = nullptr; s.list_cap = 0;
        if ((e = cudaMalloc(&s.lists, list_bytes)) != cudaSuccess) return e;
        s.list_cap = list_bytes;
    }
    if (!s.ctrs && (e = cudaMalloc(&s.ctrs, sizeof(Ctrs))) != cudaSuccess) return e;
    if (s.jobs_cap < njobs * sizeof(MixJob)) {
        if (s.jobs) cudaFree(s.jobs);
        s.jobs = nullptr; s.jobs_cap = 0;
        if ((e = cudaMalloc(&s.jobs, njobs * sizeof(MixJob))) != cudaSuccess) return e;
        s.jobs_cap = njobs * sizeof(MixJob);
    }
    if (!s.ev[0]) { cudaEventCreate(&s.ev[0]); cudaEventCreate(&s.ev[1]); }
    if ((e = cudaMemcpyAsync(s.jobs, jobs, njobs * sizeof(MixJob), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    const MixBatch mb = make_mix_batch(b);
    // launches needed: every live ion has at most min(max_more, max_steps) steps left
    const uint64_t need = max_more < b.max_steps ? (uint64_t)max_more : (uint64_t)b.max_steps;
    if (need == 0) return cudaSuccess;
    const uint32_t chunk = t.chunk ? t.chunk : 4096;
    const uint32_t full = (uint32_t)((need + chunk - 1) / chunk);
    const uint32_t launches = (t.max_launches && t.max_launches < full) ? t.max_launches : full;
    const uint32_t last_chunk = launches < full ? chunk : (uint32_t)(need - (uint64_t)(launches - 1) * chunk);
    // working state: phase offsets (2 x u64), position / velocity double-floats (12 x f32) and the
    // staged flag (u8) of every ion
    const size_t keep_bytes = (size_t)n * (2 * sizeof(uint64_t) + 12 * sizeof(float) + 1);
    if (s.keep_cap < keep_bytes) {
        if (s.keep) cudaFree(s.keep);
        s.keep = nullptr; s.keep_cap = 0;
        if ((e = cudaMalloc(&s.keep, keep_bytes)) != cudaSuccess) return e;
        s.keep_cap = keep_bytes;
    }
    if (t.sort_cells && s.sort_cap < sort_bytes(mb, n)) {
        if (s.sort) cudaFree(s.sort);
        s.sort = nullptr; s.sort_cap = 0;
        if ((e = cudaMalloc(&s.sort, sort_bytes(mb, n))) != cudaSuccess) return e;
        s.sort_cap = sort_bytes(mb, n);
    }
    Ctrs* ctr = static_cast<Ctrs*>(s.ctrs);
    if ((e = cudaMemsetAsync(ctr, 0, sizeof(Ctrs), st)) != cudaSuccess) return e;
    uint64_t* kph = static_cast<uint64_t*>(s.keep);
    float* keep = reinterpret_cast<float*>(kph + (size_t)2 * n);
    uint8_t* staged = reinterpret_cast<uint8_t*>(keep + (size_t)12 * n);
    k_init_list<<<(n + 255) / 256, 256, 0, st>>>(io, n, static_cast<uint32_t*>(s.lists), ctr, mb, keep, kph, staged);
    info->kernel_launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // resident blocks per SM: the tuning's, except for the nearest-node kernels, which hold no
    // 8-corner cache (about 100 registers instead of 167) and run as many blocks as fit
    int blocks = t.blocks_per_sm;
    if (mb.nearest) {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pick_kernel(t, mb), t.tpb, 0) == cudaSuccess && nb > 0)
            blocks = nb;
        else
            cudaGetLastError();
    }
    cudaEventRecord(s.ev[0], st);
    uint32_t kernels = 0;
    const bool graph = t.use_graph && launches > 1;
    if (graph) {
        const uint64_t key[6] = {(uint64_t)(uintptr_t)s.lists, (uint64_t)n, launches, ((uint64_t)chunk << 32) | last_chunk,
                                 (uint64_t)(uintptr_t)io.x ^ ((uint64_t)blocks << 56) ^ ((uint64_t)t.prefetch << 60) ^
                                     ((uint64_t)t.wide << 61) ^ ((uint64_t)t.sort_cells << 63),
                                 (uint64_t)(uintptr_t)s.nodes ^ ((uint64_t)mb.legacy_coll << 62) ^ ((uint64_t)mb.nearest << 61)};
        cudaGraph_t gr = nullptr;
        if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
        enqueue_launches(s, t, blocks, mb, io, n, launches, chunk, last_chunk, st, &kernels);
        e = cudaStreamEndCapture(st, &gr);
        if (e != cudaSuccess) { if (gr) cudaGraphDestroy(gr); return e; }
        // re-use the instantiated graph when only kernel parameters changed
        bool updated = false;
        if (s.graph && std::memcmp(key, s.graph_key, sizeof(key)) == 0) {
            cudaGraphExecUpdateResultInfo ri;
            if (cudaGraphExecUpdate(s.graph, gr, &ri) == cudaSuccess) updated = true;
            else cudaGetLastError();
        }
        if (!updated) {
            if (s.graph) { cudaGraphExecDestroy(s.graph); s.graph = nullptr; }
            if ((e = cudaGraphInstantiate(&s.graph, gr, 0)) != cudaSuccess) { cudaGraphDestroy(gr); return e; }
            std::memcpy(s.graph_key, key, sizeof(key));
        }
        cudaGraphDestroy(gr);
        if ((e = cudaGraphLaunch(s.graph, st)) != cudaSuccess) return e;
        info->graph_replays = 1;
    } else {
        if ((e = enqueue_launches(s, t, blocks, mb, io, n, launches, chunk, last_chunk, st, &kernels)) != cudaSuccess) return e;
    }
    cudaEventRecord(s.ev[1], st);
    if (write_states) {
        k_unstage<<<(n + 255) / 256, 256, 0, st>>>(io, n, mb, keep, staged);
        info->kernel_launches += 1;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    Ctrs h;
    if ((e = cudaMemcpyAsync(&h, ctr, sizeof(Ctrs), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    cudaEventElapsedTime(&info->step_ms, s.ev[0], s.ev[1]);
    info->ion_steps = h.steps;
    info->cell_loads = h.cell_loads;
    info->ions_queued = h.queued;
    info->step_launches = launches;
    info->kernel_launches += kernels;
    // after the last launch the surviving list must be empty unless the step budget ran out
    const uint32_t survivors = h.count[launches & 1];
    info->survivors = survivors;
    info->watchdog = (survivors != 0 && max_more >= b.max_steps) ? 1 : 0;
    return cudaSuccess;
}

}  // namespace mqmix

MQ_CHECK_READER(mq_check_read_mixed)
