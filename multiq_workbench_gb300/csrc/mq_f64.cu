// Plain FP64 ion-trajectory kernel: one thread per ion, FP64 state, f32 field nodes
// promoted to f64, global phase tables, xorshift64 collision Monte Carlo.  It evaluates
// exactly the operations of the FP64 CPU integrator in the same order and is compiled
// with --fmad=false, so its final states equal the CPU integrator's bit for bit.
//
// Reference: advance_with_field / fields_at / collide / is_crash
// (simulation/mqviz/src/world.rs:265-314,471-536) with chsim's switches
// (simulation/chsim/src/channel.metal:56-62,100-121; channel.rs:397-426).
//
// Also here: device injection (Ion::inject, world.rs:407-422), phase tables
// (Clock::fill, world.rs:445-465), the combined DC field (Fields::dc_field,
// channel.rs:220-226) and the per-job summary (summarize, channel.rs:496-506).
#include "mq_internal.h"
#include "mq_check.h"

namespace mqd {
namespace {

using mqp::Batch;
using mqp::JobC;

__global__ void k_inject(Batch b, JobTable jt, DevIons io, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // job of ion i: last job with first <= i
    uint32_t lo = 0, hi = jt.njobs;   // invariant first[lo] <= i < first[hi]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (jt.first[mid] <= i) lo = mid; else hi = mid;
    }
    uint64_t q = (uint64_t)i - jt.first[lo];
    uint64_t seed = mqp::splitmix(jt.seed[lo] + q * 0x9E37ull);
    mqp::Ion0 o;
    mqp::inject_one(b, jt.jc[lo], seed, &o);
    io.x[i] = o.x[0]; io.y[i] = o.x[1]; io.z[i] = o.x[2];
    io.vx[i] = o.v[0]; io.vy[i] = o.v[1]; io.vz[i] = o.v[2];
    io.ph_rf[i] = o.ph_rf; io.ph_ac[i] = o.ph_ac; io.rng[i] = o.rng; io.leg[i] = o.leg;
    io.steps[i] = 0; io.ncoll[i] = 0; io.status[i] = 0; io.jid[i] = lo;
}

__global__ void k_phase_table(double w, uint32_t len, double2* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    double s, c;
    mqp::phase_at(w, i, &s, &c);
    out[i] = make_double2(s, c);
}

// Comparisons and integer <-> double conversions of the step on the integer pipe. GB300's FP64 pipe
// limits this kernel and also executes FP64 compares and conversions; these helpers give the same
// results from the doubles' bit patterns (IEEE doubles of one sign order like their bits as
// integers), NaN and signed zeros included.
__device__ __forceinline__ bool is_nan_bits(long long b) { return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL; }
// x > c for a constant c > 0
__device__ __forceinline__ bool gt_pos(long long x, long long c) { return x > c && x <= 0x7FF0000000000000LL; }
// x < c for a constant c > 0 (negative numbers and -0 included, NaN excluded)
__device__ __forceinline__ bool lt_pos(long long x, long long c) { return x < c && !is_nan_bits(x); }
// x < 0
__device__ __forceinline__ bool lt_zero(long long x) { return x < 0 && x != (long long)0x8000000000000000ULL && !is_nan_bits(x); }
// mqp::cell_lo (clamp to [0, n - 2], truncate) from the bits of g; lim = the bits of (double)(n - 2)
__device__ __forceinline__ int32_t cell_lo_bits(double g, int32_t n, long long lim) {
    const long long b = __double_as_longlong(g);
    if (b <= 0 || b > 0x7FF0000000000000LL) return 0;   // !(g > 0): zeros, negatives, NaN
    if (b >= lim) return n - 2;                          // g >= n - 2, +inf included
    const int e = (int)(b >> 52) - 1023;                 // 0 < g < n - 2 < 2^31
    if (e < 0) return 0;
    return (int32_t)(((b & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL) >> (52 - e));
}
// (double)v for 0 <= v < 2^31, exactly
__device__ __forceinline__ double i2d_bits(int32_t v) {
    if (v == 0) return 0.0;
    const int e = 31 - __clz(v);
    const unsigned long long m = ((unsigned long long)(uint32_t)v << (52 - e)) & 0xFFFFFFFFFFFFFULL;
    return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | m));
}

__device__ __forceinline__ void table_get(const double2* t, uint32_t tlen, double w, uint32_t n, double* s, double* c) {
    if (n < tlen) { double2 v = __ldg(t + n); *s = v.x; *c = v.y; }
    else mqp::phase_at(w, n, s, c);
}

__global__ void __launch_bounds__(128) k_f64_step(DevGrid g, Batch b, const JobC* __restrict__ jobs,
                                                  const double2* __restrict__ rf_tab, const double2* __restrict__ ac_tab,
                                                  uint32_t tlen, DevIons io, uint32_t n, uint32_t max_more,
                                                  unsigned long long* d_steps, uint32_t* d_live) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t done = 0;
    int32_t status = 1;
    if (i < n && io.status[i] == 0) {
        const JobC jc = jobs[io.jid[i]];
        const double2* tac = ac_tab + (size_t)jc.tab * tlen;
        double x[3] = {io.x[i], io.y[i], io.z[i]};
        double v[3] = {io.vx[i], io.vy[i], io.vz[i]};
        uint64_t rng = io.rng[i];
        uint32_t age = io.steps[i], ncoll = io.ncoll[i];
        int32_t leg = io.leg[i];
        status = 0;
        double rs, rc, as_, ac;
        mqp::sincos2pi(io.ph_rf[i], &rs, &rc);
        mqp::sincos2pi(io.ph_ac[i], &as_, &ac);
        const double dt = b.dt, qmdt = jc.qmdt, h = g.h;
        // bit patterns of the step's positive thresholds for the integer-pipe comparisons
        const long long lim_x = __double_as_longlong((double)(g.nx - 2)), lim_y = __double_as_longlong((double)(g.ny - 2)),
                        lim_z = __double_as_longlong((double)(g.nz - 2));
        const long long k_exit = __double_as_longlong(b.z_exit), k_return = __double_as_longlong(b.z_return);
        const long long k_lim0 = __double_as_longlong(b.lim[0]), k_lim1 = __double_as_longlong(b.lim[1]),
                        k_lim2 = __double_as_longlong(b.lim[2]);
        const size_t nx = (size_t)g.nx, ny = (size_t)g.ny;
        while (done < max_more) {
            double S, Cc, Sa = 0.0, Ca = 0.0;
            table_get(rf_tab, tlen, b.w_rf, age, &S, &Cc);
            double srf = b.v_rf * (S * rc + Cc * rs);
            double sac = 0.0;
            if (jc.use_ac) {
                table_get(tac, tlen, jc.w_ac, age, &Sa, &Ca);
                sac = jc.v_ac * (Sa * ac + Ca * as_);
            }
            // fields_at: one pass over the 8 corners, weights (1-t, t) in order i, j, k
            double gx = mqp::div_rn(x[0], h, g.inv_h), gy = mqp::div_rn(x[1], h, g.inv_h), gz = mqp::div_rn(x[2], h, g.inv_h);
            int32_t ci = cell_lo_bits(gx, g.nx, lim_x), cj = cell_lo_bits(gy, g.ny, lim_y), ck = cell_lo_bits(gz, g.nz, lim_z);
            double tx = gx - i2d_bits(ci), ty = gy - i2d_bits(cj), tz = gz - i2d_bits(ck);
            if (b.nearest) { tx = 0.0; ty = 0.0; tz = 0.0; }
            double er[3] = {0.0, 0.0, 0.0}, ea[3] = {0.0, 0.0, 0.0}, ed[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int di = 0; di < 2; ++di) {
                double wx = di ? tx : 1.0 - tx;
#pragma unroll
                for (int dj = 0; dj < 2; ++dj) {
                    double wy = dj ? ty : 1.0 - ty;
#pragma unroll
                    for (int dk = 0; dk < 2; ++dk) {
                        double wz = dk ? tz : 1.0 - tz;
                        size_t q = (size_t)(ci + di) + nx * ((size_t)(cj + dj) + ny * (size_t)(ck + dk));
                        q = MQ_CHK(q, nx * ny * (size_t)g.nz, MQ_SITE_F64_FIELD);
                        double w = wx * wy * wz;
                        float4 r = __ldg(g.rf + q), a = __ldg(g.ac + q), c = __ldg(g.dc + q);
                        er[0] += w * mqp::widen(r.x); er[1] += w * mqp::widen(r.y); er[2] += w * mqp::widen(r.z);
                        ea[0] += w * mqp::widen(a.x); ea[1] += w * mqp::widen(a.y); ea[2] += w * mqp::widen(a.z);
                        ed[0] += w * mqp::widen(c.x); ed[1] += w * mqp::widen(c.y); ed[2] += w * mqp::widen(c.z);
                    }
                }
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                v[d] += qmdt * (srf * er[d] + sac * ea[d] + ed[d]);
                x[d] += v[d] * dt;
            }
            age += 1;
            done += 1;
            if (!b.legacy_coll) {
                double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                double bound = vm + 6.0 * jc.s_gas;
                if (mqp::xs_next(&rng) < jc.nsd * bound) {
                    double vg[3];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        double u1 = mqp::xs_next(&rng), u2 = mqp::xs_next(&rng);
                        vg[d] = jc.s_gas * mqp::gauss(u1, u2);
                    }
                    double gv[3] = {v[0] - vg[0], v[1] - vg[1], v[2] - vg[2]};
                    double gl = sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
                    if (mqp::xs_next(&rng) * bound < gl) {
                        double c = 2.0 * mqp::xs_next(&rng) - 1.0;
                        double sp, cp;
                        mqp::sincos2pi(mqp::xs_next(&rng), &sp, &cp);
                        double omc = 1.0 - c * c;
                        double sn = sqrt(omc > 0.0 ? omc : 0.0);
                        double nn[3] = {sn * cp, sn * sp, c};
#pragma unroll
                        for (int d = 0; d < 3; ++d) v[d] = v[d] - jc.mr * gv[d] + jc.mr * gl * nn[d];
                        ncoll += 1;
                    }
                }
            } else {
                leg -= 1;
                if (leg <= 0) {
                    double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    if (vm > jc.floor_v) {
                        double c = 2.0 * mqp::xs_next(&rng) - 1.0;
                        double sp, cp;
                        mqp::sincos2pi(mqp::xs_next(&rng), &sp, &cp);
                        double omc = 1.0 - c * c;
                        double sn = sqrt(omc > 0.0 ? omc : 0.0);
                        double dd[3] = {sn * cp, sn * sp, c};
                        double k1 = 1.0 - jc.mr, k2 = jc.mr * vm;
#pragma unroll
                        for (int d = 0; d < 3; ++d) v[d] = v[d] * k1 + k2 * dd[d];
                        ncoll += 1;
                    }
                    double u = mqp::xs_next(&rng);
                    double mfp = -mqp::log_(u > 1e-7 ? u : 1e-7) * jc.mfp_mean;
                    double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    double st = floor(mfp / (vn > 1e-3 ? vn : 1e-3) / dt);
                    if (st < 1.0) st = 1.0;
                    leg = !(st < 2147483647.0) ? 2147483647 : (int32_t)st;
                }
            }
            const long long bx = __double_as_longlong(x[0]), by = __double_as_longlong(x[1]), bz = __double_as_longlong(x[2]);
            if (gt_pos(bz, k_exit)) { status = 3; break; }
            if (lt_pos(bz, k_return)) { status = 2; break; }
            if (lt_zero(bx) || lt_zero(by) || lt_zero(bz) || gt_pos(bx, k_lim0) || gt_pos(by, k_lim1) || gt_pos(bz, k_lim2)) {
                status = 4;
                break;
            }
            if (x[2] > b.crash_z0 && x[2] < b.crash_z1) {
                int32_t ni = mqp::node_round(mqp::div_rn(x[0], h, g.inv_h), g.nx), nj = mqp::node_round(mqp::div_rn(x[1], h, g.inv_h), g.ny),
                        nk = mqp::node_round(mqp::div_rn(x[2], h, g.inv_h), g.nz);
                size_t q = (size_t)ni + nx * ((size_t)nj + ny * (size_t)nk);
                q = MQ_CHK(q, nx * ny * (size_t)g.nz, MQ_SITE_F64_CRASH);
                if (__ldg(&g.rf[q].w) > 0.5f) { status = 1; break; }
            }
            if (age >= b.max_steps) { status = 5; break; }
        }
        io.x[i] = x[0]; io.y[i] = x[1]; io.z[i] = x[2];
        io.vx[i] = v[0]; io.vy[i] = v[1]; io.vz[i] = v[2];
        io.rng[i] = rng; io.steps[i] = age; io.ncoll[i] = ncoll; io.leg[i] = leg; io.status[i] = status;
    }
    // warp-aggregated step and live counters
    unsigned long long s = done;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    uint32_t live = __popc(__ballot_sync(0xffffffffu, status == 0));
    if ((threadIdx.x & 31) == 0) {
        if (s) atomicAdd(d_steps, s);
        if (live) atomicAdd(d_live, live);
    }
}

__global__ void k_dc_combine(const float4* b0, const float4* b1, const float4* b2, const float4* b3,
                             float v0, float v1, float v2, float v3, float4* out, size_t n) {
    size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    // e[d] += (v[b] as f32) * dc[b][n][d], bases in order (channel.rs:223); explicit
    // round-to-nearest multiply and add keep it a two-rounding sequence like the host.
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    const float4* B[4] = {b0, b1, b2, b3};
    const float V[4] = {v0, v1, v2, v3};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!B[k]) continue;
        float4 e = B[k][q];
        ex = __fadd_rn(ex, __fmul_rn(V[k], e.x));
        ey = __fadd_rn(ey, __fmul_rn(V[k], e.y));
        ez = __fadd_rn(ez, __fmul_rn(V[k], e.z));
    }
    out[q] = make_float4(ex, ey, ez, 0.0f);
}

__global__ void k_summarize(DevIons io, uint32_t n, uint32_t njobs, unsigned long long* cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t j = io.jid[i];
    if (j >= njobs) return;
    int32_t st = io.status[i];
    int slot = st == 1 ? 0 : st == 2 ? 1 : st == 3 ? 2 : st == 4 ? 3 : 4;
    unsigned long long* c = cnt + (size_t)j * kCounters;
    atomicAdd(c + slot, 1ull);
    atomicAdd(c + 5, 1ull);
    atomicAdd(c + 6, (unsigned long long)io.ncoll[i]);
    atomicAdd(c + 7, (unsigned long long)io.steps[i]);
}

inline unsigned blocks_for(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

cudaError_t launch_inject(const mqp::Batch& b, JobTable jt, DevIons io, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_inject<<<blocks_for(n, 128), 128, 0, s>>>(b, jt, io, n);
    return cudaGetLastError();
}

cudaError_t launch_f64_step(DevGrid g, const mqp::Batch& b, const mqp::JobC* jc, const double2* rf_tab,
                            const double2* ac_tab, uint32_t tlen, DevIons io, uint32_t n, uint32_t max_more,
                            unsigned long long* d_steps, uint32_t* d_live, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_f64_step<<<blocks_for(n, 128), 128, 0, s>>>(g, b, jc, rf_tab, ac_tab, tlen, io, n, max_more, d_steps, d_live);
    return cudaGetLastError();
}

cudaError_t launch_phase_table(double w, uint32_t len, double2* out, cudaStream_t s) {
    if (len == 0) return cudaSuccess;
    k_phase_table<<<blocks_for(len, 256), 256, 0, s>>>(w, len, out);
    return cudaGetLastError();
}

cudaError_t launch_dc_combine(const float4* b0, const float4* b1, const float4* b2, const float4* b3,
                              float v0, float v1, float v2, float v3, float4* out, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_dc_combine<<<blocks_for(n, 256), 256, 0, s>>>(b0, b1, b2, b3, v0, v1, v2, v3, out, n);
    return cudaGetLastError();
}

cudaError_t launch_summarize(DevIons io, uint32_t n, uint32_t njobs, unsigned long long* counters, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_summarize<<<blocks_for(n, 256), 256, 0, s>>>(io, n, njobs, counters);
    return cudaGetLastError();
}

}  // namespace mqd

MQ_CHECK_READER(mq_check_read_f64)
