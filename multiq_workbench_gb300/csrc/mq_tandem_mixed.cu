// Mixed-precision tandem engine for sm_103a: the nine-channel transport of
// trapsim::Model::advance (simulation/trapsim/src/lib.rs:176-385) with the batched engine's
// arithmetic (FP32 fields and kinematics, compensated FP32 position and velocity).
//
//   * every launch advances all live tracks by one chunk of global steps; a bucket pass first
//     groups the tracks by region (splitter, nine ports, combiner), so warps start out
//     reading one field grid (ragged batching by field id) and lost / finished tracks drop out;
//   * position and velocity are FP32 double-floats in grid units of the track's current region
//     (cube grid in mm, or the port's grid); trapsim's enter / leave transforms (lib.rs:338-385)
//     are affine maps between the grids' coordinates, applied in double-float arithmetic with
//     double-float constants, and a port is left through the plane its double-float z crossed, so
//     the step kernel does no FP64 arithmetic (GB300's FP64 pipe made the FP64 conversions a third
//     of the pipe time in the chunks where most tracks change region);
//   * fields as interleaved node records: cube {RF, region DC} 32 B (one 256-bit load), port
//     {RF, DC (+ gate bias on idle ports), AC} 48 B with the cell's conductor bits in a spare word
//     (64-byte port records with 256-bit loads measured 28% slower: the port grids' reloads reach
//     HBM and pay for the larger footprint); the 8 corners of the track's cell are held in
//     registers and reloaded on a cell change;
//   * drive values per global step from the FP64 engine's drive table, rounded to FP32; thermal
//     collisions with Philox-4x32-10 keyed by the track key and the global step (all lanes
//     share the global step, so the generator runs warp-uniformly), their candidates drawn
//     against the majorant |v| + E|V| of mqx::thermal_partner (the reference's |v| + 6 s_gas
//     samples the same process with 2 to 3.4 times as many candidates);
//   * cube losses by the geometry test in FP32, skipped in the interior box where every
//     face is farther than the post tops (geometry.rs:166 makes such points free).
#include <cmath>
#include <cstring>
#include <vector>

#include "mq_cube_geom.h"
#include "mq_phys.h"
#include "mq_tandem_internal.h"
#include "mq_check.h"
#include "mq_mixmath.h"

namespace mqtm {
namespace {

using namespace mqx;

constexpr unsigned FULL = 0xffffffffu;
constexpr int R_SPLIT = 0, R_COMBINE = 10, R_LOST = 11;
constexpr int kNC = 21;        // counters per port
constexpr int kBuckets = 11;   // live regions 0..10
constexpr double Z_EXIT = 18.6e-3, Z_RETURN = 0.5e-3;   // world.rs:21-22
constexpr uint32_t kChunk = 256;                        // global steps per launch

// ---------------------------------------------------------------- constants
struct CubeF {   // cube geometry in mm, growth 0 (geometry.rs:136-205)
    float size, c0, pitch, half_d, t_pcb, gap, ptd, stem_r, clear_r, rod_hole, l_ext, cap_reach, cap_r, ap_r;
    int32_t n, array, ent_axis, ent_side, ent_cell0, ent_cell1, ext_axis, ext_side, ext_cell0, ext_cell1;
};

struct PortM {
    const float4* rec;       // 48 B records: {RF.xyz, 0} {DC.xyz (+ gate bias), cell conductor bits} {AC.xyz, 0}
    int32_t nx, ny, nz, idle;
    float lim[3];            // n - 1: the box of is_crash in grid units
    float pad;
    float u2v, inv_h;        // h / dt [m/s per cell/step], 1 / h [1/m]
    float zret, zexit;       // Z_RETURN / h, Z_EXIT / h
    double h, inv_hd;        // [m], 1 / h
    double u2v_d, v2u_d;     // h / dt, dt / h (region changes convert with products, not divisions)
};

struct TMConst {
    CubeF G;
    const float4* crec[2];   // cube 32 B records {RF.xyz, 0} {DC.xyz, 0}: [0] splitter, [1] combiner
    int32_t cn[3], pad0;
    float clo[3], ch;        // grid origin and spacing [mm]
    float cu2v, cinv_h;      // cube h / dt, 1 / h [1/m]
    float seam_mm, lext_mm, ent_b, ent_c;   // entrance axis centre: along z, along x [mm]
    float mouth_mm[9][2];
    double clo_d[3], ch_d, seam_m, axis_m, mouth_m[9][2];
    double clo_m[3], ch_m, inv_ch_m, cu2v_d, cv2u_d;   // cube origin and spacing [m], 1 / h, h / dt, dt / h
    PortM port[9];
    // Region changes as double-float affine maps of grid coordinates, y = a x + b per axis (the same a
    // scales the velocity): entering port i from the splitter (b[2]) or the combiner (b[3], z and its
    // velocity reversed), and leaving it through the return plane (b[2]) or the exit plane (b[3], z
    // reversed); zr / ze are the port's return / exit planes in its grid units
    float2 en_a[9], en_b[9][4], lv_a[9], lv_b[9][4], zr[9], ze[9];
    float qmdt2[8], nsd[8], mr[8];   // per species: q/m dt^2 [m per V/m], n sigma dt, M/(m+M)
    float s_gas, pad1;
    double dt;
};

struct MTracks {   // mixed-precision track state (structure of arrays)
    float *xh, *xl, *uh, *ul;   // [3][n] each
    int32_t *region, *last, *sp;
    uint64_t* key;
};

// ---------------------------------------------------------------- cube geometry in FP32
__device__ __forceinline__ float latf(const CubeF& G, int i) { return G.c0 + G.pitch * (float)i; }
__device__ __forceinline__ int round_idxf(float v, int hi) {   // v.round() as usize, clamped (NaN -> 0)
    const float r = roundf(v);
    if (!(r > 0.0f)) return 0;
    return r < (float)hi ? (int)r : hi;
}
__device__ __forceinline__ int nearest_portf(const CubeF& G, float x, float y) {   // geometry.rs:118-125
    if (!G.array) return 0;
    const float first = 0.5f * (latf(G, 2) + latf(G, 3));
    return round_idxf((x - first) / (2.0f * G.pitch), 2) + 3 * round_idxf((y - first) / (2.0f * G.pitch), 2);
}
__device__ __forceinline__ float hypf2(float u, float v) { return sqrtf(fmaf(u, u, v * v)); }

// any electrode at p (mm)?  (classify(p, 0) != FREE, geometry.rs:136-205)
__device__ bool solid(const CubeF& G, const float p[3]) {
    const float l = G.size;
    const bool inside = p[0] >= -1e-12f && p[0] <= l + 1e-12f && p[1] >= -1e-12f && p[1] <= l + 1e-12f &&
                        p[2] >= -1e-12f && p[2] <= l + 1e-12f;
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        for (int side = 0; side < 2; ++side) {
            const float u = side == 0 ? p[a] : l - p[a];
            int pid = 0, pc0 = 0, pc1 = 0;
            if (G.ent_axis == a && G.ent_side == side) { pid = 3; pc0 = G.ent_cell0; pc1 = G.ent_cell1; }
            else if (G.ext_axis == a && G.ext_side == side) {
                pid = 4;
                if (G.array) { const int i = nearest_portf(G, p[b], p[c]); pc0 = 2 + 2 * (i % 3); pc1 = 2 + 2 * (i / 3); }
                else { pc0 = G.ext_cell0; pc1 = G.ext_cell1; }
            }
            const float cb = 0.5f * (latf(G, pc0) + latf(G, pc0 + 1)), cc = 0.5f * (latf(G, pc1) + latf(G, pc1 + 1));
            if (u < 0.0f || (pid != 0 && u < 1e-12f)) {   // outside the wall: port rods and end cap
                if (pid != 0) {
                    if (u <= -G.cap_reach && hypf2(p[b] - cb, p[c] - cc) < G.cap_r) return true;
                    if (u >= -G.l_ext)
                        for (int m = 0; m < 4; ++m)
                            if (hypf2(p[b] - latf(G, pc0 + (m >> 1)), p[c] - latf(G, pc1 + (m & 1))) < G.half_d) return true;
                }
                continue;
            }
            if (!inside || u > G.ptd) continue;
            const int ib = round_idxf((p[b] - G.c0) / G.pitch, G.n - 1), ic = round_idxf((p[c] - G.c0) / G.pitch, G.n - 1);
            int idx[3];
            idx[a] = side == 0 ? 0 : G.n - 1;
            idx[b] = ib;
            idx[c] = ic;
            bool valid = true;   // post_valid (geometry.rs:81-86): idx[a] is on this face already
            for (int a2 = a + 1; a2 < 3; ++a2)
                if (idx[a2] == 0 || idx[a2] == G.n - 1) valid = false;
            const float dd = hypf2(p[b] - latf(G, ib), p[c] - latf(G, ic));
            const bool rod = pid != 0 && valid && (unsigned)(ib - pc0) <= 1u && (unsigned)(ic - pc1) <= 1u;
            const bool aperture = pid != 0 && hypf2(p[b] - cb, p[c] - cc) < G.ap_r;
            if (rod && dd < G.half_d) return true;
            if (u <= G.t_pcb && !(aperture || (valid && dd < (rod ? G.rod_hole : G.clear_r)))) return true;
            if (valid && !rod) {
                if (u <= G.t_pcb + G.gap && dd < G.stem_r) return true;
                if (u >= G.t_pcb + G.gap && dd < G.half_d) return true;
            }
        }
    }
    return false;
}

// ---------------------------------------------------------------- fields
__device__ __forceinline__ float lerp3(const float F[8], float tx, float ty, float tz) {
    const float c00 = fmaf(tx, F[1] - F[0], F[0]), c10 = fmaf(tx, F[3] - F[2], F[2]);
    const float c01 = fmaf(tx, F[5] - F[4], F[4]), c11 = fmaf(tx, F[7] - F[6], F[6]);
    const float c0 = fmaf(ty, c10 - c00, c00), c1 = fmaf(ty, c11 - c01, c01);
    return fmaf(tz, c1 - c0, c0);
}


// Register cache of the track's cell: the 8 corners x {RF, DC, AC} of its region's grid,
// reloaded only when the track changes cell or region (cube cells leave A unused).
struct TCell {
    float R[3][8], D[3][8], A[3][8];   // corner q = a + 2b + 4c
    int32_t ci, cj, ck, reg;
    float fci, fcj, fck;                // the cell as floats (no int -> float conversion per step)
    uint32_t mask;                      // port: conductor bit per corner
    uint32_t fills_cube, fills_port;    // cache fills of this lane (cube: 8 x 32-byte records; port: 8 x 48)
};

// Constants of the track's current region, held in registers and refreshed only when the track
// changes region (indexing the parameter block by region every step costs a slow indexed
// constant load per access).
struct RegK {
    const float4* rec;            // node records of the region's grid
    int32_t nx, ny, nz;
    float kick, u2v;              // q/m dt^2 / h, h / dt
    float lim0, lim1, lim2;       // port box n - 1 (grid units)
    float zret, zexit;            // port return / exit planes (grid units)
    bool cube, idle;
};

__device__ __forceinline__ void region_consts(const TMConst& C, int reg, float qmdt2, RegK& k) {
    k.cube = reg == R_SPLIT || reg == R_COMBINE;
    if (k.cube) {
        k.rec = C.crec[reg == R_COMBINE ? 1 : 0];
        k.nx = C.cn[0]; k.ny = C.cn[1]; k.nz = C.cn[2];
        k.kick = qmdt2 * C.cinv_h;
        k.u2v = C.cu2v;
        k.idle = false;
    } else {
        const PortM& P = C.port[reg - 1];
        k.rec = P.rec;
        k.nx = P.nx; k.ny = P.ny; k.nz = P.nz;
        k.kick = qmdt2 * P.inv_h;
        k.u2v = P.u2v;
        k.lim0 = P.lim[0]; k.lim1 = P.lim[1]; k.lim2 = P.lim[2];
        k.zret = P.zret; k.zexit = P.zexit;
        k.idle = P.idle != 0;
    }
}


// the cell of grid position x (clamped to the grid), reloading the cache when it changes; a change
// is found on floored floats, and indices are formed only when one is seen
__device__ __forceinline__ void cell_for(const RegK& k, int reg, const float xh[3], TCell& c) {
    if (reg == c.reg && floorf(xh[0]) == c.fci && floorf(xh[1]) == c.fcj && floorf(xh[2]) == c.fck) return;
    const int ci = clampi(__float2int_rd(xh[0]), 0, k.nx - 2), cj = clampi(__float2int_rd(xh[1]), 0, k.ny - 2),
              ck = clampi(__float2int_rd(xh[2]), 0, k.nz - 2);
    if (ci != c.ci || cj != c.cj || ck != c.ck || reg != c.reg) {
        // 32-bit record offsets (the host refuses grids with 3 x nodes >= 2^32)
        const uint32_t sy = (uint32_t)k.nx, sz = (uint32_t)k.nx * (uint32_t)k.ny;
        const uint32_t base = (uint32_t)ci + sy * (uint32_t)cj + sz * (uint32_t)ck;
        uint32_t m = 0;
        if (k.cube) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                uint32_t o = 2u * (base + (uint32_t)(q & 1) + ((q & 2) ? sy : 0u) + ((q & 4) ? sz : 0u));
                o = (uint32_t)MQ_CHK_SPAN(o, 2, 2 * (size_t)sz * (size_t)k.nz, MQ_SITE_TMX_CELL);
                float4 r, d;
                ld256(k.rec + o, r, d);   // a 32-byte cube record in one load (1.6% on the tandem)
                c.R[0][q] = r.x; c.R[1][q] = r.y; c.R[2][q] = r.z;
                c.D[0][q] = d.x; c.D[1][q] = d.y; c.D[2][q] = d.z;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                uint32_t o = 3u * (base + (uint32_t)(q & 1) + ((q & 2) ? sy : 0u) + ((q & 4) ? sz : 0u));
                o = (uint32_t)MQ_CHK_SPAN(o, 3, 3 * (size_t)sz * (size_t)k.nz, MQ_SITE_TMX_CELL);
                const float4 r = __ldg(k.rec + o), d = __ldg(k.rec + o + 1), a = __ldg(k.rec + o + 2);
                c.R[0][q] = r.x; c.R[1][q] = r.y; c.R[2][q] = r.z;
                c.D[0][q] = d.x; c.D[1][q] = d.y; c.D[2][q] = d.z;
                c.A[0][q] = a.x; c.A[1][q] = a.y; c.A[2][q] = a.z;
                if (q == 0) m = __float_as_uint(d.w);
            }
        }
        c.mask = m;
        if (k.cube) ++c.fills_cube; else ++c.fills_port;
        c.ci = ci; c.cj = cj; c.ck = ck; c.reg = reg;
        c.fci = (float)ci; c.fcj = (float)cj; c.fck = (float)ck;
    }
}

// y = a x + b for a double-float x = (xh, xl) and double-float constants a, b (an exact product of
// the high parts by fma, the small cross terms added to its error): about 2^-46 relative, on the
// FP32 pipe
__device__ __forceinline__ void df_affine(float xh, float xl, float2 a, float2 b, float& yh, float& yl) {
    const float p = __fmul_rn(a.x, xh);
    const float t = fmaf(a.x, xl, fmaf(a.y, xh, fmaf(a.x, xh, -p)));
    float s, e;
    two_sum(p, b.x, s, e);
    e = __fadd_rn(e, __fadd_rn(t, b.y));
    fast_two_sum(s, e, yh, yl);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// (xh + xl) < (t.x + t.y) for double-floats, exact in sign where the high parts are within a factor 2
__device__ __forceinline__ bool df_less(float xh, float xl, float2 t) {
    return __fadd_rn(__fsub_rn(xh, t.x), __fsub_rn(xl, t.y)) < 0.0f;
}

// double-float <-> FP64
__device__ __forceinline__ double ddv(float h, float l) { return (double)h + (double)l; }
__device__ __forceinline__ void splitd(double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

// FP64 physical state -> mixed state in the region's grid units
__global__ void k_tm_load(TMConst C, Tracks64 T, MTracks M, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = T.region[i];
    M.region[i] = r;
    M.last[i] = T.last[i];
    M.sp[i] = T.sp[i];
    M.key[i] = T.rng[i];
    if (r > R_COMBINE) return;
    const double x[3] = {T.x[i], T.y[i], T.z[i]}, v[3] = {T.vx[i], T.vy[i], T.vz[i]};
    for (int d = 0; d < 3; ++d) {
        double g, u;
        if (r == R_SPLIT || r == R_COMBINE) {
            g = (x[d] * 1000.0 - C.clo_d[d]) / C.ch_d;
            u = v[d] * C.dt * 1000.0 / C.ch_d;
        } else {
            g = x[d] / C.port[r - 1].h;
            u = v[d] * C.dt / C.port[r - 1].h;
        }
        splitd(g, M.xh[(size_t)d * n + i], M.xl[(size_t)d * n + i]);
        splitd(u, M.uh[(size_t)d * n + i], M.ul[(size_t)d * n + i]);
    }
}

// mixed state -> FP64 physical state
__global__ void k_tm_store(TMConst C, Tracks64 T, MTracks M, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = M.region[i];
    T.region[i] = r;
    T.last[i] = M.last[i];
    if (r > R_COMBINE) return;   // finished tracks keep the state they left with
    double x[3], v[3];
    for (int d = 0; d < 3; ++d) {
        const double g = ddv(M.xh[(size_t)d * n + i], M.xl[(size_t)d * n + i]);
        const double u = ddv(M.uh[(size_t)d * n + i], M.ul[(size_t)d * n + i]);
        if (r == R_SPLIT || r == R_COMBINE) {
            x[d] = (C.clo_d[d] + g * C.ch_d) * 1e-3;
            v[d] = u * C.ch_d * 1e-3 / C.dt;
        } else {
            x[d] = g * C.port[r - 1].h;
            v[d] = u * C.port[r - 1].h / C.dt;
        }
    }
    T.x[i] = x[0]; T.y[i] = x[1]; T.z[i] = x[2];
    T.vx[i] = v[0]; T.vy[i] = v[1]; T.vz[i] = v[2];
}

// group the live tracks by region: list[r * n + k], one warp-aggregated atomic per region group
__global__ void k_tm_bucket(const int32_t* __restrict__ region, uint32_t n, uint32_t* __restrict__ list,
                            uint32_t* __restrict__ bcount) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = i < n ? region[i] : R_LOST;
    const bool live = r <= R_COMBINE;
    const unsigned lm = __ballot_sync(FULL, live);
    if (!live) return;
    const unsigned peers = __match_any_sync(lm, r);
    const int leader = __ffs(peers) - 1;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&bcount[r], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    list[MQ_CHK((size_t)r * n + base + __popc(peers & ((1u << lane) - 1u)), (size_t)kBuckets * n, MQ_SITE_TMX_LIST)] = i;
}

// one chunk of global steps for every live track (one thread per track, grouped by region)
__global__ void __launch_bounds__(128, 3) k_tm_step(TMConst C, MTracks M, uint32_t n, const uint32_t* __restrict__ list,
                                                    const uint32_t* __restrict__ bcount, const float* __restrict__ drive,
                                                    uint64_t g0, uint32_t S, uint32_t* __restrict__ counts,
                                                    unsigned long long* __restrict__ stepc) {
    __shared__ uint32_t off[kBuckets + 1];
    if (threadIdx.x == 0) {
        uint32_t a = 0;
        for (int r = 0; r < kBuckets; ++r) { off[r] = a; a += bcount[r]; }
        off[kBuckets] = a;
    }
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n_cube = 0, n_port = 0, n_idle = 0, f_cube = 0, f_port = 0;
    if (t < off[kBuckets]) {
        int r0 = 0;
        while (r0 < kBuckets - 1 && t >= off[r0 + 1]) ++r0;
        const uint32_t id = (uint32_t)MQ_CHK(list[(size_t)r0 * n + (t - off[r0])], n, MQ_SITE_TMX_LIST);
        int reg = r0, last = M.last[id];
        const int sp = M.sp[id];
        const uint64_t key = M.key[id];
        const uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
        float xh[3], xl[3], uh[3], ul[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            xh[d] = M.xh[(size_t)d * n + id]; xl[d] = M.xl[(size_t)d * n + id];
            uh[d] = M.uh[(size_t)d * n + id]; ul[d] = M.ul[(size_t)d * n + id];
        }
        const float qmdt2 = C.qmdt2[sp], nsd = C.nsd[sp], mr = C.mr[sp];
        RegK rk;
        region_consts(C, reg, qmdt2, rk);
        TCell c;
        c.ci = c.cj = c.ck = -1;
        c.reg = -1;
        c.fills_cube = c.fills_port = 0;
        c.fci = c.fcj = c.fck = __int_as_float(0x7fc00000);
        cell_for(rk, reg, xh, c);
        uint4 rc = make_uint4(0, 0, 0, 0);
        for (uint32_t k = 0; k < S && reg <= R_COMBINE; ++k) {
            const uint64_t g = g0 + k;
            if (k == 0 || (g & 3) == 0) rc = philox(k0, k1, (uint32_t)(g >> 2), (uint32_t)(g >> 34), 0u, 0u);
            const float* dr = drive + (size_t)k * 10;
            const float rf = __ldg(dr);
            const bool cube = rk.cube;
            float E[3];
            const float kick = rk.kick, u2v = rk.u2v;
            {
                float tx = __fadd_rn(__fsub_rn(xh[0], c.fci), xl[0]);
                float ty = __fadd_rn(__fsub_rn(xh[1], c.fcj), xl[1]);
                float tz = __fadd_rn(__fsub_rn(xh[2], c.fck), xl[2]);
                if (cube) {   // fields.rs:89-96 clamps the grid coordinate to the grid
                    tx = __saturatef(tx); ty = __saturatef(ty); tz = __saturatef(tz);
                }
                const float ac = cube ? 0.0f : __ldg(dr + reg);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    float F[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) F[q] = cube ? fmaf(rf, c.R[d][q], c.D[d][q]) : fmaf(rf, c.R[d][q], fmaf(ac, c.A[d][q], c.D[d][q]));
                    E[d] = lerp3(F, tx, ty, tz);
                }
            }
            if (cube) ++n_cube;
            else if (rk.idle) ++n_idle;
            else ++n_port;
            // kick and drift, compensated (transport_step, lib.rs:90-103)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float inc = __fadd_rn(__fmul_rn(kick, E[d]), ul[d]);
                two_sum(uh[d], inc, uh[d], ul[d]);
                float s, e;
                fast_two_sum(xh[d], uh[d], s, e);
                e = __fadd_rn(e, __fadd_rn(xl[d], ul[d]));
                fast_two_sum(s, e, xh[d], xl[d]);
            }
            // null-collision thermal bath (world.rs:473-488) with the majorant |v| + E|V| of
            // thermal_partner: candidate if u0 < nsd (|v| + E|V|)
            {
                const uint32_t q = (uint32_t)(g & 3);
                const float u0 = unif(q == 0 ? rc.x : q == 1 ? rc.y : q == 2 ? rc.z : rc.w);
                const float um2 = fmaf(uh[0], uh[0], fmaf(uh[1], uh[1], uh[2] * uh[2]));
                const float ca = nsd * u2v, du = u0 - nsd * kMeanSpeed * C.s_gas;
                if (du < 0.0f || du * du < ca * ca * um2) {
                    const uint4 r0 = philox(k0, k1, (uint32_t)g, (uint32_t)(g >> 32), 1u, 0u);
                    const uint4 r1 = philox(k0, k1, (uint32_t)g, (uint32_t)(g >> 32), 2u, 0u);
                    const float v[3] = {uh[0] * u2v, uh[1] * u2v, uh[2] * u2v};
                    float gv[3], vm_sum;
                    thermal_partner(r0, C.s_gas, sqrtf(um2) * u2v, v, gv, vm_sum);
                    const float gl = sqrtf(fmaf(gv[0], gv[0], fmaf(gv[1], gv[1], gv[2] * gv[2])));
                    if (unif16(r0.w & 0xffffu) * vm_sum < gl) {
                        const float cth = 2.0f * unif(r1.x) - 1.0f;
                        float sp_, cp_;
                        angle_sincos(unif(r1.y), &sp_, &cp_);
                        const float sn = sqrtf(fmaxf(0.0f, 1.0f - cth * cth));
                        const float nn[3] = {sn * cp_, sn * sp_, cth};
                        const float v2u = 1.0f / u2v;
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            uh[d] = fmaf(mr * gl, nn[d], fmaf(-mr, gv[d], v[d])) * v2u;
                            ul[d] = 0.0f;
                        }
                    }
                }
            }
            // routing (lib.rs:212-272)
            if (cube) {
                float p[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) p[d] = fmaf(xh[d], C.ch, fmaf(xl[d], C.ch, C.clo[d]));
                const float lo_in = C.G.ptd, hi_in = C.G.size - C.G.ptd;
                const bool interior = p[0] > lo_in && p[0] < hi_in && p[1] > lo_in && p[1] < hi_in && p[2] > lo_in &&
                                      p[2] < hi_in;
                if (!interior && solid(C.G, p)) { reg = R_LOST; continue; }
                if (p[2] > C.seam_mm) {
                    const int i = nearest_portf(C.G, p[0], p[1]);
                    if (hypf2(p[0] - C.mouth_mm[i][0], p[1] - C.mouth_mm[i][1]) < C.G.ap_r) {
                        // enter (lib.rs:338-367): straight into the port's grid units
                        uint32_t* cnt = counts + (size_t)i * kNC;
                        const bool fwd = reg == R_SPLIT;
                        const float2 a = C.en_a[i];
                        df_affine(xh[0], xl[0], a, C.en_b[i][0], xh[0], xl[0]);
                        df_affine(xh[1], xl[1], a, C.en_b[i][1], xh[1], xl[1]);
                        df_affine(xh[2], xl[2], fwd ? a : neg2(a), C.en_b[i][fwd ? 2 : 3], xh[2], xl[2]);
                        const float2 z0 = make_float2(0.0f, 0.0f);
                        df_affine(uh[0], ul[0], a, z0, uh[0], ul[0]);
                        df_affine(uh[1], ul[1], a, z0, uh[1], ul[1]);
                        df_affine(uh[2], ul[2], fwd ? a : neg2(a), z0, uh[2], ul[2]);
                        if (fwd) {
                            atomicAdd(cnt + 0, 1u);
                            if (last >= 0) {
                                atomicAdd(cnt + 3, 1u);
                                atomicAdd(cnt + 5 + last, 1u);
                                if (last != i) atomicAdd(cnt + 4, 1u);
                            }
                        } else {
                            atomicAdd(cnt + 14, 1u);
                        }
                        reg = 1 + i;
                        region_consts(C, reg, qmdt2, rk);
                        cell_for(rk, reg, xh, c);
                        continue;
                    }
                    if (p[2] > C.G.size) { reg = R_LOST; continue; }
                }
                if (p[1] > C.G.size && hypf2(p[0] - C.ent_c, p[2] - C.ent_b) >= C.G.ap_r) { reg = R_LOST; continue; }
                if (p[1] > C.G.size + C.lext_mm) reg = reg == R_SPLIT ? 12 : 13;
                else if (p[0] < 0.0f || p[1] < 0.0f || p[2] < 0.0f || p[0] > C.G.size) reg = R_LOST;
                else cell_for(rk, reg, xh, c);
            } else {
                const int i = reg - 1;
                uint32_t* cnt = counts + (size_t)i * kNC;
                // is_crash (world.rs:309-314): outside the box, or the nearest node is a conductor
                bool crash = xh[0] < 0.0f || xh[1] < 0.0f || xh[2] < 0.0f || xh[0] > rk.lim0 || xh[1] > rk.lim1 ||
                             xh[2] > rk.lim2;
                if (!crash) {
                    cell_for(rk, reg, xh, c);
                    const uint32_t qn = (__fadd_rn(__fsub_rn(xh[0], c.fci), xl[0]) >= 0.5f ? 1u : 0u) |
                                        (__fadd_rn(__fsub_rn(xh[1], c.fcj), xl[1]) >= 0.5f ? 2u : 0u) |
                                        (__fadd_rn(__fsub_rn(xh[2], c.fck), xl[2]) >= 0.5f ? 4u : 0u);
                    crash = (c.mask >> qn) & 1u;
                }
                if (crash) {
                    reg = R_LOST;
                    atomicAdd(cnt + 15, 1u);
                } else if ((xh[2] < rk.zret + 1.0f && df_less(xh[2], xl[2], C.zr[i])) ||
                           (xh[2] > rk.zexit - 1.0f && df_less(C.ze[i].x, C.ze[i].y, make_float2(xh[2], xl[2])))) {
                    // leave (lib.rs:368-385) through the plane crossed, decided on the double-float z,
                    // straight into the cube's grid units
                    const bool ret = df_less(xh[2], xl[2], C.zr[i]);
                    const float2 a = C.lv_a[i], z0 = make_float2(0.0f, 0.0f);
                    df_affine(xh[0], xl[0], a, C.lv_b[i][0], xh[0], xl[0]);
                    df_affine(xh[1], xl[1], a, C.lv_b[i][1], xh[1], xl[1]);
                    df_affine(xh[2], xl[2], ret ? a : neg2(a), C.lv_b[i][ret ? 2 : 3], xh[2], xl[2]);
                    df_affine(uh[0], ul[0], a, z0, uh[0], ul[0]);
                    df_affine(uh[1], ul[1], a, z0, uh[1], ul[1]);
                    df_affine(uh[2], ul[2], ret ? a : neg2(a), z0, uh[2], ul[2]);
                    if (ret) {
                        reg = R_SPLIT;
                        last = i;
                        atomicAdd(cnt + 1, 1u);
                    } else {
                        reg = R_COMBINE;
                        last = -1;
                        atomicAdd(cnt + 2, 1u);
                        atomicAdd(cnt + 16 + sp, 1u);
                    }
                    region_consts(C, reg, qmdt2, rk);
                    cell_for(rk, reg, xh, c);
                }
            }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            M.xh[(size_t)d * n + id] = xh[d]; M.xl[(size_t)d * n + id] = xl[d];
            M.uh[(size_t)d * n + id] = uh[d]; M.ul[(size_t)d * n + id] = ul[d];
        }
        M.region[id] = reg;
        M.last[id] = last;
        f_cube = c.fills_cube;
        f_port = c.fills_port;
    }
    // executed track-steps by region kind: one atomic per warp (every lane reaches this point)
    n_cube = __reduce_add_sync(FULL, n_cube);
    n_port = __reduce_add_sync(FULL, n_port);
    n_idle = __reduce_add_sync(FULL, n_idle);
    f_cube = __reduce_add_sync(FULL, f_cube);
    f_port = __reduce_add_sync(FULL, f_port);
    if ((threadIdx.x & 31) == 0) {
        if (n_cube) atomicAdd(stepc + 0, (unsigned long long)n_cube);
        if (n_port) atomicAdd(stepc + 1, (unsigned long long)n_port);
        if (n_idle) atomicAdd(stepc + 2, (unsigned long long)n_idle);
        if (f_cube) atomicAdd(stepc + 3, (unsigned long long)f_cube);
        if (f_port) atomicAdd(stepc + 4, (unsigned long long)f_port);
    }
}

// cube records: {RF.xyz, 0} {DC_region.xyz, 0}
__global__ void k_tm_pack_cube(const float4* __restrict__ rf, const float4* __restrict__ dc, float4* __restrict__ rec,
                               size_t nodes) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nodes) return;
    const float4 r = rf[q], d = dc[q];
    rec[2 * q] = make_float4(r.x, r.y, r.z, 0.0f);
    rec[2 * q + 1] = make_float4(d.x, d.y, d.z, 0.0f);
}

// port records: {RF.xyz, 0} {DC.xyz + bias * gate.xyz, conductor bits of the cell} {AC.xyz, 0}
__global__ void k_tm_pack_port(const float4* __restrict__ rf, const float4* __restrict__ ac, const float4* __restrict__ dc,
                               const float4* __restrict__ gate, float bias, int32_t nx, int32_t ny, int32_t nz,
                               float4* __restrict__ rec) {
    const size_t nodes = (size_t)nx * ny * nz;
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nodes) return;
    const float4 r = rf[q], d = dc[q], a = ac[q];
    const float4 gt = bias != 0.0f ? gate[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    const size_t sy = (size_t)nx, sz = (size_t)nx * (size_t)ny;
    const int32_t i = (int32_t)(q % sy), j = (int32_t)((q / sy) % (size_t)ny), k = (int32_t)(q / sz);
    uint32_t m = 0;
    if (i < nx - 1 && j < ny - 1 && k < nz - 1)
        for (int c = 0; c < 8; ++c)
            m |= (rf[q + (size_t)(c & 1) + ((c & 2) ? sy : 0) + ((c & 4) ? sz : 0)].w > 0.5f ? 1u : 0u) << c;
    rec[3 * q] = make_float4(r.x, r.y, r.z, 0.0f);
    rec[3 * q + 1] = make_float4(fmaf(bias, gt.x, d.x), fmaf(bias, gt.y, d.y), fmaf(bias, gt.z, d.z), __uint_as_float(m));
    rec[3 * q + 2] = make_float4(a.x, a.y, a.z, 0.0f);
}

}  // namespace

struct State {
    TMConst C;
    std::vector<void*> allocs;
    MTracks M{};
    uint32_t cap = 0;
    uint32_t* list = nullptr;
    uint32_t* bcount = nullptr;
};

static void free_tracks(State* s) {
    for (void* p : {(void*)s->M.xh, (void*)s->M.xl, (void*)s->M.uh, (void*)s->M.ul, (void*)s->M.region, (void*)s->M.last,
                    (void*)s->M.sp, (void*)s->M.key, (void*)s->list})
        if (p) cudaFree(p);
    s->M = MTracks{};
    s->list = nullptr;
    s->cap = 0;
}

State* create(const mq_tandem_desc& d, const DevFields& f, cudaStream_t st, std::string& err) {
    State* s = new (std::nothrow) State();
    if (!s) { err = "out of host memory"; return nullptr; }
    std::memset(&s->C, 0, sizeof(s->C));
    TMConst& C = s->C;
    auto fail = [&](const char* what, cudaError_t e) -> State* {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        destroy(s);
        return nullptr;
    };
    cudaError_t e;
    // cube geometry in FP32 (growth 0)
    const mq_cube_geom& g = d.cube;
    CubeF& G = C.G;
    G.size = (float)mqc::size(g);
    G.c0 = (float)mqc::c0(g);
    G.pitch = (float)g.pitch;
    G.half_d = (float)(g.d / 2.0);
    G.t_pcb = (float)g.t_pcb;
    G.gap = (float)g.gap;
    G.ptd = (float)mqc::post_top_depth(g);
    G.stem_r = (float)g.stem_r;
    G.clear_r = (float)g.clear_r;
    G.rod_hole = (float)(g.d / 2.0 + g.rod_clear_extra);
    G.l_ext = (float)g.l_ext;
    G.cap_reach = (float)(g.l_ext + g.cap_gap);
    G.cap_r = (float)g.cap_r;
    G.ap_r = (float)g.ap_r;
    G.n = g.n; G.array = g.array;
    G.ent_axis = g.ent_axis; G.ent_side = g.ent_side; G.ent_cell0 = g.ent_cell[0]; G.ent_cell1 = g.ent_cell[1];
    G.ext_axis = g.ext_axis; G.ext_side = g.ext_side; G.ext_cell0 = g.ext_cell[0]; G.ext_cell1 = g.ext_cell[1];
    // cube grid and the two region DC sets
    const size_t cn = (size_t)d.cube_dims[0] * d.cube_dims[1] * d.cube_dims[2];
    if (3 * cn >= ((size_t)1 << 32)) return fail("cube grid too large for 32-bit record offsets", cudaErrorInvalidValue);
    for (int a = 0; a < 3; ++a) {
        C.cn[a] = d.cube_dims[a];
        C.clo[a] = (float)d.cube_lo_mm[a];
        C.clo_d[a] = d.cube_lo_mm[a];
    }
    C.ch = (float)d.cube_h_mm;
    C.ch_d = d.cube_h_mm;
    for (int a = 0; a < 3; ++a) C.clo_m[a] = d.cube_lo_mm[a] * 1e-3;
    C.ch_m = d.cube_h_mm * 1e-3;
    C.inv_ch_m = 1.0 / C.ch_m;
    C.cu2v_d = C.ch_m / d.dt;
    C.cv2u_d = d.dt / C.ch_m;
    C.cu2v = (float)(d.cube_h_mm * 1e-3 / d.dt);
    C.cinv_h = (float)(1.0 / (d.cube_h_mm * 1e-3));
    for (int r = 0; r < 2; ++r) {
        void* p = nullptr;
        if ((e = cudaMalloc(&p, cn * 32)) != cudaSuccess) return fail("cube records", e);
        s->allocs.push_back(p);
        C.crec[r] = static_cast<const float4*>(p);
        k_tm_pack_cube<<<(unsigned)((cn + 255) / 256), 256, 0, st>>>(f.crf, f.cdc[r], static_cast<float4*>(p), cn);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail("cube pack", e);
    }
    // layout: seam, mouths, entrance axis
    double seam = 0, size = 0, mouths[18], ent[2];
    mq_tandem_layout(&d, &seam, &size, mouths);
    mq_cube_port_axis(&d.cube, -1, ent);
    C.seam_m = seam;
    C.seam_mm = (float)(seam * 1000.0);
    C.lext_mm = (float)g.l_ext;
    C.ent_b = (float)ent[0];
    C.ent_c = (float)ent[1];
    C.axis_m = d.ch_axis_mm * 1e-3;
    for (int i = 0; i < 9; ++i)
        for (int k = 0; k < 2; ++k) {
            C.mouth_m[i][k] = mouths[2 * i + k];
            C.mouth_mm[i][k] = (float)(mouths[2 * i + k] * 1000.0);
        }
    // region-change maps (enter: lib.rs:338-367, leave: lib.rs:368-385) in grid coordinates
    auto df = [](double v) { const float h = (float)v; return make_float2(h, (float)(v - (double)h)); };
    for (int i = 0; i < 9; ++i) {
        const double hp = d.port[i].h, hc = C.ch_m;
        const double dx = C.axis_m - C.mouth_m[i][0], dy = C.axis_m - C.mouth_m[i][1];
        C.en_a[i] = df(hc / hp);
        C.en_b[i][0] = df((C.clo_m[0] + dx) / hp);
        C.en_b[i][1] = df((C.clo_m[1] + dy) / hp);
        C.en_b[i][2] = df((Z_RETURN + C.clo_m[2] - C.seam_m) / hp);   // from the splitter
        C.en_b[i][3] = df((Z_EXIT - C.clo_m[2] + C.seam_m) / hp);     // from the combiner, z reversed
        C.lv_a[i] = df(hp / hc);
        C.lv_b[i][0] = df((-dx - C.clo_m[0]) / hc);
        C.lv_b[i][1] = df((-dy - C.clo_m[1]) / hc);
        C.lv_b[i][2] = df((C.seam_m - Z_RETURN - C.clo_m[2]) / hc);    // back to the splitter
        C.lv_b[i][3] = df((C.seam_m + Z_EXIT - C.clo_m[2]) / hc);      // on to the combiner, z reversed
        C.zr[i] = df(Z_RETURN / hp);
        C.ze[i] = df(Z_EXIT / hp);
    }
    // ports: one packed record array per distinct (grid arrays, idle)
    struct Key { const float4 *rf, *ac, *dc, *gate; int idle; const float4* rec; };
    std::vector<Key> made;
    for (int i = 0; i < 9; ++i) {
        const mq_tandem_port& tp = d.port[i];
        PortM& P = C.port[i];
        P.nx = tp.dims[0]; P.ny = tp.dims[1]; P.nz = tp.dims[2];
        for (int a = 0; a < 3; ++a) P.lim[a] = (float)(tp.dims[a] - 1);
        P.idle = tp.tone_khz == 0.0;
        P.h = tp.h;
        P.inv_hd = 1.0 / tp.h;
        P.u2v_d = tp.h / d.dt;
        P.v2u_d = d.dt / tp.h;
        P.u2v = (float)(tp.h / d.dt);
        P.inv_h = (float)(1.0 / tp.h);
        P.zret = (float)(Z_RETURN / tp.h);
        P.zexit = (float)(Z_EXIT / tp.h);
        const Key k{f.prf[i], f.pac[i], f.pdc[i], f.pgate[i], P.idle, nullptr};
        for (const Key& m : made)
            if (m.rf == k.rf && m.ac == k.ac && m.dc == k.dc && m.gate == k.gate && m.idle == k.idle) P.rec = m.rec;
        if (!P.rec) {
            const size_t nodes = (size_t)P.nx * P.ny * P.nz;
            if (3 * nodes >= ((size_t)1 << 32)) return fail("port grid too large for 32-bit record offsets", cudaErrorInvalidValue);
            void* p = nullptr;
            if ((e = cudaMalloc(&p, nodes * 48)) != cudaSuccess) return fail("port records", e);
            s->allocs.push_back(p);
            k_tm_pack_port<<<(unsigned)((nodes + 255) / 256), 256, 0, st>>>(f.prf[i], f.pac[i], f.pdc[i], f.pgate[i],
                                                                            P.idle ? (float)d.gate_bias_v : 0.0f, P.nx,
                                                                            P.ny, P.nz, static_cast<float4*>(p));
            if ((e = cudaGetLastError()) != cudaSuccess) return fail("port pack", e);
            P.rec = static_cast<const float4*>(p);
            Key km = k;
            km.rec = P.rec;
            made.push_back(km);
        }
    }
    // species (SpPhys::new, world.rs:342-347) and the gas
    const double mg = 28.0 * mqp::AMU;
    const double ngas = d.pressure_pa / (mqp::KB * d.temp_k);
    C.s_gas = (float)std::sqrt(mqp::KB * d.temp_k / mg);
    C.dt = d.dt;
    for (int k = 0; k < d.nspecies && k < 8; ++k) {
        const double m = d.species[k].mass * mqp::AMU;
        C.qmdt2[k] = (float)(d.species[k].z * mqp::QE / m * d.dt * d.dt);
        C.nsd[k] = (float)(ngas * d.species[k].ccs * 1e-20 * d.dt);
        C.mr[k] = (float)(mg / (m + mg));
    }
    if ((e = cudaMalloc(&s->bcount, kBuckets * sizeof(uint32_t))) != cudaSuccess) return fail("bucket counters", e);
    return s;
}

void destroy(State* s) {
    if (!s) return;
    free_tracks(s);
    for (void* p : s->allocs) cudaFree(p);
    if (s->bcount) cudaFree(s->bcount);
    delete s;
}

static cudaError_t reserve(State* s, uint32_t n) {
    if (s->cap >= n && s->M.xh) return cudaSuccess;
    free_tracks(s);
    cudaError_t e;
    const size_t m = n ? n : 1;
    if ((e = cudaMalloc(&s->M.xh, 3 * m * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.xl, 3 * m * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.uh, 3 * m * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.ul, 3 * m * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.region, m * sizeof(int32_t))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.last, m * sizeof(int32_t))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.sp, m * sizeof(int32_t))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->M.key, m * sizeof(uint64_t))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s->list, (size_t)kBuckets * m * sizeof(uint32_t))) != cudaSuccess) return e;
    s->cap = n;
    return cudaSuccess;
}

cudaError_t load(State* s, const Tracks64& tr, uint32_t n, cudaStream_t st, uint32_t* launches) {
    cudaError_t e = reserve(s, n);
    if (e != cudaSuccess) return e;
    if (!n) return cudaSuccess;
    k_tm_load<<<(n + 127) / 128, 128, 0, st>>>(s->C, tr, s->M, n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t store(State* s, const Tracks64& tr, uint32_t n, cudaStream_t st, uint32_t* launches) {
    if (!n) return cudaSuccess;
    k_tm_store<<<(n + 127) / 128, 128, 0, st>>>(s->C, tr, s->M, n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t run(State* s, uint32_t n, const float* drive, uint64_t step0, uint64_t k, uint32_t* counts,
                unsigned long long* stepc, cudaStream_t st, uint32_t* launches) {
    cudaError_t e;
    if (!n) return cudaSuccess;
    const unsigned grid = (n + 127) / 128;
    for (uint64_t q = 0; q < k; q += kChunk) {
        const uint32_t S = (uint32_t)(k - q < kChunk ? k - q : kChunk);
        if ((e = cudaMemsetAsync(s->bcount, 0, kBuckets * sizeof(uint32_t), st)) != cudaSuccess) return e;
        k_tm_bucket<<<grid, 128, 0, st>>>(s->M.region, n, s->list, s->bcount);
        k_tm_step<<<grid, 128, 0, st>>>(s->C, s->M, n, s->list, s->bcount, drive + q * 10, step0 + q, S, counts, stepc);
        *launches += 2;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace mqtm

MQ_CHECK_READER(mq_check_read_tandem_mixed)
