// Nine-channel tandem transport on the GPU: one thread per track, all tracks in lockstep on
// the global clock, FP64 state, compiled without FMA contraction so that every track's
// arithmetic equals the CPU restatement of trapsim::Model::advance bit for bit.
//
// Reference: simulation/trapsim/src/lib.rs:69-103 (cube_field, transport_step),
// lib.rs:176-276 (Model::advance: region fields, routing), lib.rs:338-385 (enter / leave),
// simulation/mqviz/src/world.rs:265-314 (fields_at, gate_delta, is_crash), world.rs:471-488
// (collide).
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "mq_cube_geom.h"
#include "mq_phys.h"
#include "mq_tandem.h"
#include "mq_tandem_internal.h"
#include "mq_check.h"

namespace {

constexpr double Z_EXIT = 18.6e-3;     // world.rs:21
constexpr double Z_RETURN = 0.5e-3;    // world.rs:22
constexpr int R_SPLIT = 0, R_COMBINE = 10, R_LOST = 11, R_BACK = 12, R_DETECTED = 13;
constexpr int kNC = 21;                 // counters per port (mq_port_counts)

struct TSpec { double qmdt, s_ion, mr, nsd; };

struct TPort {                  // one port's channel grid and drive
    int32_t kn[3], idle;
    double kh, inv_kh, lim[3];   // spacing [m], its correctly rounded reciprocal, box limits
    const float4 *rf, *ac, *dc, *gate;
};

struct TConst {
    mq_cube_geom cube;
    int32_t cn[3];
    double clo[3], ch_mm, inv_ch_mm;
    const float4* crf;
    const float4* cdc[2];
    TPort port[9];
    double axis, seam, size, ap_r, l_ext_m, dt, s_gas, gate_v;
    double mouth[9][2];
    double ent_b, ent_c;   // entrance axis centre (mm): along z, along x
    TSpec sp[8];
};

struct Tracks {
    double *x, *y, *z, *vx, *vy, *vz;
    uint64_t* rng;
    int32_t *sp, *region, *last;
};

__device__ __forceinline__ double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// cube_field: trilinear RF * rf + combined DC at a point (lib.rs:70-88, fields.rs:89-96)
__device__ void cube_field(const TConst& C, const float4* dc, const double x[3], double rf, double e[3]) {
    int c[3];
    double w[3];
    for (int a = 0; a < 3; ++a) {
        const double p = x[a] * 1000.0;
        const double f = clampd(mqp::div_rn(p - C.clo[a], C.ch_mm, C.inv_ch_mm), 0.0, (double)(C.cn[a] - 1) - 1e-9);
        c[a] = f > 0.0 ? (int)floor(f) : 0;   // NaN -> 0 as Rust's `as usize`
        w[a] = f - (double)c[a];
    }
    e[0] = e[1] = e[2] = 0.0;
    for (int k = 0; k < 2; ++k)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                size_t q = (size_t)(c[0] + i) + (size_t)C.cn[0] * ((size_t)(c[1] + j) + (size_t)C.cn[1] * (size_t)(c[2] + k));
                q = MQ_CHK(q, (size_t)C.cn[0] * (size_t)C.cn[1] * (size_t)C.cn[2], MQ_SITE_TDM_CUBE);
                const double wt = (i == 1 ? w[0] : 1.0 - w[0]) * (j == 1 ? w[1] : 1.0 - w[1]) * (k == 1 ? w[2] : 1.0 - w[2]);
                const float4 r = C.crf[q], d = dc[q];
                e[0] += wt * (rf * (double)r.x + (double)d.x);
                e[1] += wt * (rf * (double)r.y + (double)d.y);
                e[2] += wt * (rf * (double)r.z + (double)d.z);
            }
}

// channel fields_at (world.rs:265-288) and gate_delta (world.rs:291-302) on the port's grid
__device__ void chan_field(const TPort& P, double gate_v, const double x[3], double rf, double ac, double e[3]) {
    const double h = P.kh;
    const double g[3] = {mqp::div_rn(x[0], h, P.inv_kh), mqp::div_rn(x[1], h, P.inv_kh), mqp::div_rn(x[2], h, P.inv_kh)};
    const int32_t i0 = mqp::cell_lo(g[0], P.kn[0]), j0 = mqp::cell_lo(g[1], P.kn[1]), k0 = mqp::cell_lo(g[2], P.kn[2]);
    const double tx = g[0] - (double)i0, ty = g[1] - (double)j0, tz = g[2] - (double)k0;
    double er[3] = {0, 0, 0}, ea[3] = {0, 0, 0}, ed[3] = {0, 0, 0};
    const size_t nx = (size_t)P.kn[0], ny = (size_t)P.kn[1];
    for (int di = 0; di < 2; ++di) {
        const double wx = di ? tx : 1.0 - tx;
        for (int dj = 0; dj < 2; ++dj) {
            const double wy = dj ? ty : 1.0 - ty;
            for (int dk = 0; dk < 2; ++dk) {
                const double wz = dk ? tz : 1.0 - tz;
                size_t q = (size_t)(i0 + di) + nx * ((size_t)(j0 + dj) + ny * (size_t)(k0 + dk));
                q = MQ_CHK(q, nx * ny * (size_t)P.kn[2], MQ_SITE_TDM_PORT);
                const double w = wx * wy * wz;
                const float4 r = P.rf[q], a = P.ac[q], d = P.dc[q];
                er[0] += w * (double)r.x; er[1] += w * (double)r.y; er[2] += w * (double)r.z;
                ea[0] += w * (double)a.x; ea[1] += w * (double)a.y; ea[2] += w * (double)a.z;
                ed[0] += w * (double)d.x; ed[1] += w * (double)d.y; ed[2] += w * (double)d.z;
            }
        }
    }
    double bias[3] = {0.0, 0.0, 0.0};
    if (P.idle) {
        for (int ii = 0; ii < 2; ++ii)
            for (int jj = 0; jj < 2; ++jj)
                for (int kk = 0; kk < 2; ++kk) {
                    size_t q = (size_t)(i0 + ii) + nx * ((size_t)(j0 + jj) + ny * (size_t)(k0 + kk));
                    q = MQ_CHK(q, nx * ny * (size_t)P.kn[2], MQ_SITE_TDM_GATE);
                    const double w = gate_v * (ii == 1 ? tx : 1.0 - tx) * (jj == 1 ? ty : 1.0 - ty) * (kk == 1 ? tz : 1.0 - tz);
                    const float4 b = P.gate[q];
                    bias[0] += w * (double)b.x; bias[1] += w * (double)b.y; bias[2] += w * (double)b.z;
                }
    }
    for (int k = 0; k < 3; ++k) e[k] = rf * er[k] + ac * ea[k] + ed[k] + bias[k];
}

__device__ bool chan_crash(const TPort& P, const double x[3]) {   // world.rs:309-314
    for (int d = 0; d < 3; ++d)
        if (x[d] < 0.0 || x[d] > P.lim[d]) return true;
    const int32_t ni = mqp::node_round(mqp::div_rn(x[0], P.kh, P.inv_kh), P.kn[0]),
                  nj = mqp::node_round(mqp::div_rn(x[1], P.kh, P.inv_kh), P.kn[1]),
                  nk = mqp::node_round(mqp::div_rn(x[2], P.kh, P.inv_kh), P.kn[2]);
    size_t q = (size_t)ni + (size_t)P.kn[0] * ((size_t)nj + (size_t)P.kn[1] * (size_t)nk);
    q = MQ_CHK(q, (size_t)P.kn[0] * (size_t)P.kn[1] * (size_t)P.kn[2], MQ_SITE_TDM_CRASH);
    return P.rf[q].w > 0.5f;
}

__device__ void collide(double v[3], uint64_t* rng, const TSpec& s, double s_gas) {   // world.rs:473-488
    const double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double bound = vm + 6.0 * s_gas;
    if (mqp::xs_next(rng) < s.nsd * bound) {
        double vg[3];
        for (int d = 0; d < 3; ++d) {
            const double u1 = mqp::xs_next(rng), u2 = mqp::xs_next(rng);
            vg[d] = s_gas * mqp::gauss(u1, u2);
        }
        const double gv[3] = {v[0] - vg[0], v[1] - vg[1], v[2] - vg[2]};
        const double gl = sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
        if (mqp::xs_next(rng) * bound < gl) {
            const double c = 2.0 * mqp::xs_next(rng) - 1.0;
            double sp, cp;
            mqp::sincos2pi(mqp::xs_next(rng), &sp, &cp);
            const double omc = 1.0 - c * c;
            const double sn = sqrt(omc > 0.0 ? omc : 0.0);
            const double nn[3] = {sn * cp, sn * sp, c};
            for (int d = 0; d < 3; ++d) v[d] = v[d] - s.mr * gv[d] + s.mr * gl * nn[d];
        }
    }
}

// Executed track-steps by region kind (cube, driven port, idle port): one warp-reduced atomic per warp.
__device__ __forceinline__ void add_steps(unsigned long long* st, uint32_t c, uint32_t p, uint32_t q) {
    c = __reduce_add_sync(0xffffffffu, c);
    p = __reduce_add_sync(0xffffffffu, p);
    q = __reduce_add_sync(0xffffffffu, q);
    if ((threadIdx.x & 31) == 0) {
        if (c) atomicAdd(st + 0, (unsigned long long)c);
        if (p) atomicAdd(st + 1, (unsigned long long)p);
        if (q) atomicAdd(st + 2, (unsigned long long)q);
    }
}

// blockDim.x is a multiple of 32 and no lane returns early, so the warp reductions see full warps.
__global__ void __launch_bounds__(128) k_tandem(TConst C, Tracks T, uint32_t n, const double* __restrict__ drive,
                                                uint32_t steps, uint32_t* __restrict__ counts,
                                                unsigned long long* __restrict__ stepc) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n_cube = 0, n_port = 0, n_idle = 0;
    if (id < n && T.region[id] < R_LOST) {
        int reg = T.region[id];
        double x[3] = {T.x[id], T.y[id], T.z[id]};
        double v[3] = {T.vx[id], T.vy[id], T.vz[id]};
        uint64_t rng = T.rng[id];
        const int sp = T.sp[id];
        int last = T.last[id];
        const TSpec S = C.sp[sp];
        for (uint32_t k = 0; k < steps && reg < R_LOST; ++k) {
            const double* dr = drive + (size_t)k * 10;   // rf, ac[0..9)
            const double rf = dr[0];
            double e[3];
            if (reg == R_SPLIT || reg == R_COMBINE) {
                cube_field(C, C.cdc[reg == R_COMBINE ? 1 : 0], x, rf, e);
                ++n_cube;
            } else {
                const int i = reg - 1;
                chan_field(C.port[i], C.gate_v, x, rf, dr[1 + i], e);
                if (C.port[i].idle) ++n_idle;
                else ++n_port;
            }
            // transport_step (lib.rs:90-103)
            for (int d = 0; d < 3; ++d) {
                v[d] += S.qmdt * e[d];
                x[d] += v[d] * C.dt;
            }
            collide(v, &rng, S, C.s_gas);
            if (reg == R_SPLIT || reg == R_COMBINE) {
                const double mm[3] = {x[0] * 1000.0, x[1] * 1000.0, x[2] * 1000.0};
                int sg = 0;
                if (mqc::classify(C.cube, mm, 0.0, &sg) != mqc::ID_FREE) { reg = R_LOST; continue; }
                if (x[2] > C.seam) {
                    const int i = mqc::nearest_port(C.cube, mm[0], mm[1]);
                    const double* c = C.mouth[i];
                    if (mqc::dist2d(x[0] - c[0], x[1] - c[1]) < C.ap_r * 0.001) {
                        // enter (lib.rs:338-367)
                        uint32_t* cnt = counts + (size_t)i * kNC;
                        x[0] += C.axis - c[0];
                        x[1] += C.axis - c[1];
                        const double depth = x[2] - C.seam;
                        if (reg == R_SPLIT) {
                            x[2] = Z_RETURN + depth;
                            atomicAdd(cnt + 0, 1u);
                            if (last >= 0) {
                                atomicAdd(cnt + 3, 1u);
                                atomicAdd(cnt + 5 + last, 1u);
                                if (last != i) atomicAdd(cnt + 4, 1u);
                            }
                        } else {
                            x[2] = Z_EXIT - depth;
                            v[2] *= -1.0;
                            atomicAdd(cnt + 14, 1u);
                        }
                        reg = 1 + i;
                        continue;
                    }
                    if (x[2] > C.size) { reg = R_LOST; continue; }
                }
                if (x[1] > C.size) {
                    if (mqc::dist2d(mm[0] - C.ent_c, mm[2] - C.ent_b) >= C.ap_r) { reg = R_LOST; continue; }
                }
                if (x[1] > C.size + C.l_ext_m) reg = (reg == R_SPLIT) ? R_BACK : R_DETECTED;
                else if (x[0] < 0.0 || x[1] < 0.0 || x[2] < 0.0 || x[0] > C.size) reg = R_LOST;
            } else {
                const int i = reg - 1;
                uint32_t* cnt = counts + (size_t)i * kNC;
                if (chan_crash(C.port[i], x)) { reg = R_LOST; atomicAdd(cnt + 15, 1u); }
                else if (x[2] < Z_RETURN || x[2] > Z_EXIT) {
                    // leave (lib.rs:368-385)
                    const double* c = C.mouth[i];
                    x[0] += c[0] - C.axis;
                    x[1] += c[1] - C.axis;
                    if (x[2] < Z_RETURN) {
                        x[2] = C.seam + x[2] - Z_RETURN;
                        reg = R_SPLIT;
                        last = i;
                        atomicAdd(cnt + 1, 1u);
                    } else {
                        x[2] = C.seam - (x[2] - Z_EXIT);
                        v[2] *= -1.0;
                        reg = R_COMBINE;
                        last = -1;
                        atomicAdd(cnt + 2, 1u);
                        atomicAdd(cnt + 16 + sp, 1u);
                    }
                }
            }
        }
        T.x[id] = x[0]; T.y[id] = x[1]; T.z[id] = x[2];
        T.vx[id] = v[0]; T.vy[id] = v[1]; T.vz[id] = v[2];
        T.rng[id] = rng; T.region[id] = reg; T.last[id] = last;
    }
    add_steps(stepc, n_cube, n_port, n_idle);
}

}  // namespace

struct mq_tandem {
    int dev = 0;
    std::string err;
    mq_tandem_desc desc;
    TConst C;
    std::vector<std::pair<const float*, void*>> bufs;   // host array -> device copy (shared arrays uploaded once)
    void* tr = nullptr;
    size_t tr_cap = 0;
    void* drive = nullptr;
    size_t drive_cap = 0;
    uint32_t* counts = nullptr;
    unsigned long long* stepc = nullptr;   // executed track-steps: cube, driven port, idle port; mixed engine's
                                           // cell-cache fills: cube, port
    mqtm::State* mix = nullptr;            // the mixed-precision engine (MQ_PREC_MIXED)
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace {
mq_status tfail(mq_tandem* t, mq_status c, const std::string& m) {
    if (t) t->err = m;
    return c;
}
#define TCK(call, what) do { cudaError_t c_ = (call); if (c_ != cudaSuccess) return tfail(t, c_ == cudaErrorMemoryAllocation ? MQ_ERR_NOMEM : MQ_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(c_)); } while (0)

// drive of global steps [s0, s0 + k): rf = V_rf sin(2 pi f_rf t), ac_i = V_ac sin(2 pi f_i t), t = s dt (lib.rs:178-182)
void drive_table(const mq_tandem_desc& d, uint64_t s0, uint64_t k, double* out) {
    for (uint64_t q = 0; q < k; ++q) {
        const double t = (double)(s0 + q) * d.dt;
        double s, c;
        double p = d.f_rf * t;
        mqp::sincos2pi(p - floor(p), &s, &c);
        out[10 * q] = d.v_rf * s;
        for (int i = 0; i < 9; ++i) {
            p = d.port[i].tone_khz * 1000.0 * t;
            mqp::sincos2pi(p - floor(p), &s, &c);
            out[10 * q + 1 + i] = d.port[i].v_ac * s;
        }
    }
}
}  // namespace

extern "C" {

mq_status mq_tandem_create(const mq_tandem_desc* d, int32_t device, mq_tandem** out) {
    if (!out) return MQ_ERR_INVALID;
    *out = nullptr;
    if (!d || !d->cube_rf4 || !d->cube_dc4[0] || !d->cube_dc4[1] || d->nspecies < 1 ||
        d->nspecies > 5 || !(d->dt > 0) || !(d->cube_h_mm > 0) ||   // five charge-state counters per port
        (d->precision != MQ_PREC_F64 && d->precision != MQ_PREC_MIXED))
        return MQ_ERR_INVALID;
    for (int a = 0; a < 3; ++a)
        if (d->cube_dims[a] < 2) return MQ_ERR_INVALID;
    for (const mq_tandem_port& p : d->port) {
        if (!p.rf4 || !p.ac4 || !p.dc4 || !p.gate4 || !(p.h > 0)) return MQ_ERR_INVALID;
        for (int a = 0; a < 3; ++a)
            if (p.dims[a] < 2) return MQ_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) { cudaGetLastError(); return MQ_ERR_NO_DEVICE; }
    mq_tandem* t = new (std::nothrow) mq_tandem();
    if (!t) return MQ_ERR_NOMEM;
    t->dev = device;
    t->desc = *d;
    auto bail = [&](mq_status s) { mq_tandem_destroy(t); return s; };
    if (cudaSetDevice(device) != cudaSuccess) return bail(MQ_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) != cudaSuccess) return bail(MQ_ERR_CUDA);
    for (auto& e : t->ev) if (cudaEventCreate(&e) != cudaSuccess) return bail(MQ_ERR_CUDA);
    // upload a node array (float4 per node) unless the same host array is already resident
    auto upload = [&](const float* src, size_t nodes, const float4** dst) -> bool {
        for (auto& b : t->bufs)
            if (b.first == src) { *dst = static_cast<const float4*>(b.second); return true; }
        void* p = nullptr;
        if (cudaMalloc(&p, nodes * 16) != cudaSuccess) return false;
        t->bufs.emplace_back(src, p);
        if (cudaMemcpy(p, src, nodes * 16, cudaMemcpyHostToDevice) != cudaSuccess) return false;
        *dst = static_cast<const float4*>(p);
        return true;
    };
    TConst& C = t->C;
    std::memset(&C, 0, sizeof(C));
    const size_t cn = (size_t)d->cube_dims[0] * d->cube_dims[1] * d->cube_dims[2];
    if (!upload(d->cube_rf4, cn, &C.crf) || !upload(d->cube_dc4[0], cn, &C.cdc[0]) || !upload(d->cube_dc4[1], cn, &C.cdc[1]))
        return bail(MQ_ERR_NOMEM);
    for (int i = 0; i < 9; ++i) {
        const mq_tandem_port& p = d->port[i];
        TPort& P = C.port[i];
        const size_t kn = (size_t)p.dims[0] * p.dims[1] * p.dims[2];
        if (!upload(p.rf4, kn, &P.rf) || !upload(p.ac4, kn, &P.ac) || !upload(p.dc4, kn, &P.dc) || !upload(p.gate4, kn, &P.gate))
            return bail(MQ_ERR_NOMEM);
        for (int a = 0; a < 3; ++a) {
            P.kn[a] = p.dims[a];
            P.lim[a] = (double)(p.dims[a] - 1) * p.h;   // World::lim (world.rs:145)
        }
        P.kh = p.h;
        P.inv_kh = 1.0 / p.h;
        P.idle = p.tone_khz == 0.0;
    }
    if (cudaMalloc(&t->counts, 9 * kNC * sizeof(uint32_t)) != cudaSuccess) return bail(MQ_ERR_NOMEM);
    if (cudaMalloc(&t->stepc, 5 * sizeof(unsigned long long)) != cudaSuccess) return bail(MQ_ERR_NOMEM);
    C.cube = d->cube;
    for (int a = 0; a < 3; ++a) { C.cn[a] = d->cube_dims[a]; C.clo[a] = d->cube_lo_mm[a]; }
    C.ch_mm = d->cube_h_mm;
    C.inv_ch_mm = 1.0 / d->cube_h_mm;
    double mouths[18];
    mq_tandem_layout(d, &C.seam, &C.size, mouths);
    for (int i = 0; i < 9; ++i) { C.mouth[i][0] = mouths[2 * i]; C.mouth[i][1] = mouths[2 * i + 1]; }
    double ent[2];
    mq_cube_port_axis(&d->cube, -1, ent);
    C.ent_b = ent[0]; C.ent_c = ent[1];
    C.axis = d->ch_axis_mm * 1e-3;
    C.ap_r = d->cube.ap_r;
    C.l_ext_m = d->cube.l_ext * 0.001;
    C.dt = d->dt;
    C.gate_v = d->gate_bias_v;
    const double mg = 28.0 * mqp::AMU;
    const double ngas = d->pressure_pa / (mqp::KB * d->temp_k);
    C.s_gas = sqrt(mqp::KB * d->temp_k / mg);
    for (int s = 0; s < d->nspecies; ++s) {   // SpPhys::new (world.rs:342-347)
        const double m = d->species[s].mass * mqp::AMU;
        const double qm = d->species[s].z * mqp::QE / m;
        C.sp[s].qmdt = qm * d->dt;
        C.sp[s].s_ion = sqrt(mqp::KB * d->temp_k / m);
        C.sp[s].mr = mg / (m + mg);
        C.sp[s].nsd = (ngas * (d->species[s].ccs * 1e-20)) * d->dt;
    }
    if (d->precision == MQ_PREC_MIXED) {
        mqtm::DevFields f;
        f.crf = C.crf;
        f.cdc[0] = C.cdc[0];
        f.cdc[1] = C.cdc[1];
        for (int i = 0; i < 9; ++i) {
            f.prf[i] = C.port[i].rf; f.pac[i] = C.port[i].ac; f.pdc[i] = C.port[i].dc; f.pgate[i] = C.port[i].gate;
        }
        std::string err;
        t->mix = mqtm::create(*d, f, t->st, err);
        if (!t->mix) { mq_tandem_destroy(t); return MQ_ERR_NOMEM; }
        if (cudaStreamSynchronize(t->st) != cudaSuccess) return bail(MQ_ERR_CUDA);
    }
    *out = t;
    return MQ_OK;
}

void mq_tandem_destroy(mq_tandem* t) {
    if (!t) return;
    cudaSetDevice(t->dev);
    if (t->st) cudaStreamSynchronize(t->st);
    for (auto& b : t->bufs) cudaFree(b.second);
    if (t->tr) cudaFree(t->tr);
    if (t->drive) cudaFree(t->drive);
    if (t->counts) cudaFree(t->counts);
    if (t->stepc) cudaFree(t->stepc);
    if (t->mix) mqtm::destroy(t->mix);
    for (auto& e : t->ev) if (e) cudaEventDestroy(e);
    if (t->st) cudaStreamDestroy(t->st);
    delete t;
}

const char* mq_tandem_last_error(mq_tandem* t) { return t ? t->err.c_str() : "null tandem"; }

mq_status mq_tandem_advance(mq_tandem* t, mq_tracks* tr, size_t n, uint64_t step0, uint64_t steps, mq_port_counts counts[9],
                            mq_tandem_stats* stats) {
    if (!t || !tr || !counts) return MQ_ERR_INVALID;
    if (n > 0xFFFFFFF0ull) return tfail(t, MQ_ERR_TOO_LARGE, "at most 2^32-16 tracks");
    TCK(cudaSetDevice(t->dev), "cudaSetDevice");
    const size_t tb = n * (7 * 8 + 3 * 4);
    if (t->tr_cap < tb) {
        if (t->tr) cudaFree(t->tr);
        t->tr = nullptr; t->tr_cap = 0;
        TCK(cudaMalloc(&t->tr, tb ? tb : 16), "track buffers");
        t->tr_cap = tb;
    }
    char* base = static_cast<char*>(t->tr);
    Tracks T;
    void* host[10] = {tr->x, tr->y, tr->z, tr->vx, tr->vy, tr->vz, tr->rng, tr->sp, tr->region, tr->last};
    const size_t sz[10] = {8, 8, 8, 8, 8, 8, 8, 4, 4, 4};
    void* dev[10];
    size_t off = 0;
    for (int k = 0; k < 10; ++k) {
        if (!host[k]) return tfail(t, MQ_ERR_INVALID, "track array missing");
        dev[k] = base + off;
        off += sz[k] * n;
    }
    T.x = (double*)dev[0]; T.y = (double*)dev[1]; T.z = (double*)dev[2];
    T.vx = (double*)dev[3]; T.vy = (double*)dev[4]; T.vz = (double*)dev[5];
    T.rng = (uint64_t*)dev[6]; T.sp = (int32_t*)dev[7]; T.region = (int32_t*)dev[8]; T.last = (int32_t*)dev[9];
    const mqtm::Tracks64 T64{T.x, T.y, T.z, T.vx, T.vy, T.vz, T.rng, T.sp, T.region, T.last};
    for (size_t i = 0; i < n; ++i)   // the kernel indexes species constants and counters by these
        if (tr->sp[i] < 0 || tr->sp[i] >= t->desc.nspecies || tr->region[i] < 0 || tr->region[i] > R_DETECTED ||
            tr->last[i] < -1 || tr->last[i] > 8)
            return tfail(t, MQ_ERR_INVALID, "track " + std::to_string(i) + " has an invalid species, region or last port");
    for (int k = 0; k < 10; ++k) TCK(cudaMemcpyAsync(dev[k], host[k], sz[k] * n, cudaMemcpyHostToDevice, t->st), "track upload");
    std::vector<uint32_t> cnt(9 * kNC);
    for (int i = 0; i < 9; ++i) std::memcpy(&cnt[(size_t)i * kNC], &counts[i], sizeof(mq_port_counts));
    TCK(cudaMemcpyAsync(t->counts, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, t->st), "counter upload");
    TCK(cudaMemsetAsync(t->stepc, 0, 5 * sizeof(unsigned long long), t->st), "step counters");
    // Drive table: up to kTab steps per upload; kernels of `per` steps each, about 2^27 track-steps
    // per launch so that no single launch runs for long.
    const uint64_t kTab = 65536;
    const uint64_t tab = steps < kTab ? (steps ? steps : 1) : kTab;
    if (t->drive_cap < tab * 10 * 8) {
        if (t->drive) cudaFree(t->drive);
        t->drive = nullptr; t->drive_cap = 0;
        TCK(cudaMalloc(&t->drive, tab * 10 * 8), "drive table");
        t->drive_cap = tab * 10 * 8;
    }
    uint64_t per = n ? ((uint64_t)1 << 27) / n : tab;
    per = per < 32 ? 32 : (per > 4096 ? 4096 : per);
    std::vector<double> dtab(tab * 10);
    std::vector<float> ftab(t->mix ? tab * 10 : 0);
    uint32_t launches = 0;
    uint64_t h2d = tb + cnt.size() * 4;
    for (uint64_t s = 0; s < steps || s == 0; s += tab) {
        const uint64_t k = steps - s < tab ? steps - s : tab;
        drive_table(t->desc, step0 + s, k, dtab.data());
        // pageable source: the call returns once the host buffer has been staged, so it may be refilled next
        if (t->mix) {   // the mixed engine reads the drive as FP32 (no FP64 conversions in its step loop)
            for (uint64_t q = 0; q < k * 10; ++q) ftab[q] = (float)dtab[q];
            if (k) TCK(cudaMemcpyAsync(t->drive, ftab.data(), k * 10 * 4, cudaMemcpyHostToDevice, t->st), "drive upload");
            h2d += k * 10 * 4;
        } else {
            if (k) TCK(cudaMemcpyAsync(t->drive, dtab.data(), k * 10 * 8, cudaMemcpyHostToDevice, t->st), "drive upload");
            h2d += k * 10 * 8;
        }
        if (s == 0) {
            TCK(cudaEventRecord(t->ev[0], t->st), "event");   // times the kernels (and later table blocks)
            if (t->mix) TCK(mqtm::load(t->mix, T64, (uint32_t)n, t->st, &launches), "mixed tandem load");
        }
        if (!steps) break;
        if (t->mix) {
            TCK(mqtm::run(t->mix, (uint32_t)n, (const float*)t->drive, step0 + s, k, t->counts, t->stepc, t->st, &launches),
                "mixed tandem kernel");
            continue;
        }
        for (uint64_t q = 0; q < k && n; q += per, ++launches) {
            const uint64_t m = k - q < per ? k - q : per;
            k_tandem<<<(unsigned)((n + 127) / 128), 128, 0, t->st>>>(t->C, T, (uint32_t)n, (const double*)t->drive + q * 10,
                                                                    (uint32_t)m, t->counts, t->stepc);
            TCK(cudaGetLastError(), "tandem kernel");
        }
    }
    if (t->mix) TCK(mqtm::store(t->mix, T64, (uint32_t)n, t->st, &launches), "mixed tandem store");
    TCK(cudaEventRecord(t->ev[1], t->st), "event");
    for (int k = 0; k < 10; ++k) TCK(cudaMemcpyAsync(host[k], dev[k], sz[k] * n, cudaMemcpyDeviceToHost, t->st), "track download");
    TCK(cudaMemcpyAsync(cnt.data(), t->counts, cnt.size() * 4, cudaMemcpyDeviceToHost, t->st), "counter download");
    unsigned long long sc[5] = {0, 0, 0, 0, 0};
    TCK(cudaMemcpyAsync(sc, t->stepc, sizeof(sc), cudaMemcpyDeviceToHost, t->st), "step counters");
    TCK(cudaStreamSynchronize(t->st), "tandem");
    for (int i = 0; i < 9; ++i) std::memcpy(&counts[i], &cnt[(size_t)i * kNC], sizeof(mq_port_counts));
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t->ev[0], t->ev[1]);
        std::memset(stats, 0, sizeof(*stats));
        stats->steps_cube = sc[0];
        stats->steps_port = sc[1];
        stats->steps_idle = sc[2];
        stats->cell_fills_cube = sc[3];
        stats->cell_fills_port = sc[4];
        stats->kernel_ms = ms;
        stats->launches = launches;
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = tb + cnt.size() * 4 + sizeof(sc);
    }
    return MQ_OK;
}

}  // extern "C"

MQ_CHECK_READER(mq_check_read_tandem)
