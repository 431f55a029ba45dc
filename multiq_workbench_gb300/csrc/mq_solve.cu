// Device Laplace solver: the host solver of mq_grid.cpp (conjugate gradients preconditioned by a
// symmetric geometric V-cycle with red-black Gauss-Seidel smoothing, stopping on the scaled
// max-norm residual) run on the GPU with the same arithmetic in the same order, so the two give
// bit-identical potentials: every node update is the host's expression (this unit is compiled
// without FMA contraction), a colour's nodes are independent within a half sweep, and the dot
// products are summed row by row, plane by plane, exactly as the host sums them.
//
// Replaces the set-up step before the path (fieldsolve's solve, simulation/fieldsolve/src/lib.rs:164,
// as restated by mq_laplace_solve) where grids of 10^7-10^8 nodes make the host solve the cost.
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "mq_grid.h"
#include "mq_levels.h"

namespace {

constexpr int kT = 256;

struct DLevel {
    int nx, ny, nz;
    uint8_t* fix;
    double *u, *rhs, *r;
    size_t n() const { return (size_t)nx * ny * nz; }
};

__global__ void k_gs(double* __restrict__ u, const double* __restrict__ rhs, const uint8_t* __restrict__ fix, int nx,
                     int ny, int nz, int col) {
    const int hx = (nx - 1) / 2;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)hx * (ny - 2) * (nz - 2)) return;
    const int m = (int)(t % hx);
    const size_t r = t / hx;
    const int j = 1 + (int)(r % (ny - 2)), k = 1 + (int)(r / (ny - 2));
    const int i = 1 + ((1 + j + k + col) & 1) + 2 * m;
    if (i > nx - 2) return;
    const size_t sy = nx, sz = (size_t)nx * ny;
    const size_t q = (size_t)i + sy * j + sz * k;
    if (fix[q]) return;
    const double s = u[q - 1] + u[q + 1] + u[q - sy] + u[q + sy] + u[q - sz] + u[q + sz];
    u[q] = (rhs[q] + s) / 6.0;
}

// the coarsest level: sweeps x (red, black, black, red) in one block
__global__ void k_coarse(double* __restrict__ u, const double* __restrict__ rhs, const uint8_t* __restrict__ fix, int nx,
                         int ny, int nz, int sweeps) {
    const int hx = (nx - 1) / 2;
    const int total = hx * (ny - 2) * (nz - 2);
    const size_t sy = nx, sz = (size_t)nx * ny;
    for (int s = 0; s < sweeps; ++s)
        for (int h = 0; h < 4; ++h) {
            const int col = (h == 0 || h == 3) ? 0 : 1;
            for (int t = threadIdx.x; t < total; t += blockDim.x) {
                const int m = t % hx, r = t / hx;
                const int j = 1 + r % (ny - 2), k = 1 + r / (ny - 2);
                const int i = 1 + ((1 + j + k + col) & 1) + 2 * m;
                if (i > nx - 2) continue;
                const size_t q = (size_t)i + sy * j + sz * k;
                if (fix[q]) continue;
                const double v = u[q - 1] + u[q + 1] + u[q - sy] + u[q + sy] + u[q - sz] + u[q + sz];
                u[q] = (rhs[q] + v) / 6.0;
            }
            __syncthreads();
        }
}

__global__ void k_residual(const double* __restrict__ u, const double* __restrict__ rhs, const uint8_t* __restrict__ fix,
                           double* __restrict__ r, int nx, int ny, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    if (fix[q]) { r[q] = 0.0; return; }
    const size_t sy = nx, sz = (size_t)nx * ny;
    const double s = u[q - 1] + u[q + 1] + u[q - sy] + u[q + sy] + u[q - sz] + u[q + sz];
    r[q] = rhs[q] + s - 6.0 * u[q];
}

__global__ void k_restrict(const double* __restrict__ fr, int fnx, int fny, int fnz, double* __restrict__ crhs,
                           const uint8_t* __restrict__ cfix, int cnx, int cny, int cnz) {
    const size_t qc = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qc >= (size_t)cnx * cny * cnz) return;
    if (cfix[qc]) { crhs[qc] = 0.0; return; }
    const int I = (int)(qc % cnx), J = (int)((qc / cnx) % cny), K = (int)(qc / ((size_t)cnx * cny));
    double s = 0.0;
    for (int dk = -1; dk <= 1; ++dk) {
        const int k = 2 * K + dk;
        if (k < 0 || k >= fnz) continue;
        const double wk = dk == 0 ? 1.0 : 0.5;
        for (int dj = -1; dj <= 1; ++dj) {
            const int j = 2 * J + dj;
            if (j < 0 || j >= fny) continue;
            const double wj = dj == 0 ? 1.0 : 0.5;
            for (int di = -1; di <= 1; ++di) {
                const int i = 2 * I + di;
                if (i < 0 || i >= fnx) continue;
                const double wi = di == 0 ? 1.0 : 0.5;
                s += (wk * wj * wi) * fr[(size_t)i + (size_t)fnx * ((size_t)j + (size_t)fny * k)];
            }
        }
    }
    crhs[qc] = 0.5 * s;
}

__global__ void k_prolong(const double* __restrict__ cu, int cnx, int cny, double* __restrict__ fu,
                          const uint8_t* __restrict__ ffix, int fnx, int fny, int fnz) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (size_t)fnx * fny * fnz) return;
    if (ffix[q]) return;
    const int i = (int)(q % fnx), j = (int)((q / fnx) % fny), k = (int)(q / ((size_t)fnx * fny));
    const int k0 = k / 2, k1 = (k + 1) / 2, j0 = j / 2, j1 = (j + 1) / 2, i0 = i / 2, i1 = (i + 1) / 2;
    const double wk1 = (k & 1) ? 0.5 : 0.0, wk0 = (k & 1) ? 0.5 : 1.0;
    const double wj1 = (j & 1) ? 0.5 : 0.0, wj0 = (j & 1) ? 0.5 : 1.0;
    const double wi1 = (i & 1) ? 0.5 : 0.0, wi0 = (i & 1) ? 0.5 : 1.0;
    auto c = [&](int a, int b, int d) { return cu[(size_t)a + (size_t)cnx * ((size_t)b + (size_t)cny * d)]; };
    double s = 0.0;
    s += wk0 * wj0 * wi0 * c(i0, j0, k0);
    if (wi1 != 0.0) s += wk0 * wj0 * wi1 * c(i1, j0, k0);
    if (wj1 != 0.0) {
        s += wk0 * wj1 * wi0 * c(i0, j1, k0);
        if (wi1 != 0.0) s += wk0 * wj1 * wi1 * c(i1, j1, k0);
    }
    if (wk1 != 0.0) {
        s += wk1 * wj0 * wi0 * c(i0, j0, k1);
        if (wi1 != 0.0) s += wk1 * wj0 * wi1 * c(i1, j0, k1);
        if (wj1 != 0.0) {
            s += wk1 * wj1 * wi0 * c(i0, j1, k1);
            if (wi1 != 0.0) s += wk1 * wj1 * wi1 * c(i1, j1, k1);
        }
    }
    fu[q] += s;
}

// max |x| of non-negative doubles: their bit patterns order like the values
__device__ __forceinline__ void max_into(unsigned long long* m, double v) {
    if (v == v) atomicMax(m, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// r = S-residual of phi at free nodes (sum of neighbours - 6 phi), 0 at fixed; max |r|
__global__ void k_true_residual(const double* __restrict__ phi, const uint8_t* __restrict__ fix, double* __restrict__ r,
                                int nx, int ny, size_t n, unsigned long long* __restrict__ rmax) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0;
    if (q < n) {
        if (fix[q]) r[q] = 0.0;
        else {
            const size_t sy = nx, sz = (size_t)nx * ny;
            const double s = phi[q - 1] + phi[q + 1] + phi[q - sy] + phi[q + sy] + phi[q - sz] + phi[q + sz];
            r[q] = s - 6.0 * phi[q];
            a = fabs(r[q]);
        }
    }
    a = warp_max(a);
    if ((threadIdx.x & 31) == 0) max_into(rmax, a);
}

// per row (j, k): sum over i of a[q] * b[q], in i order
__global__ void k_row_dot(const double* __restrict__ a, const double* __restrict__ b, int nx, size_t rows,
                          double* __restrict__ rowsum) {
    const size_t row = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    const size_t base = row * (size_t)nx;
    double s = 0.0;
    for (int i = 0; i < nx; ++i) s += a[base + i] * b[base + i];
    rowsum[row] = s;
}

// per row: q = S p at free nodes (0 at fixed) and the row's sum of p[q] * q[q], in i order
__global__ void k_row_sp(const double* __restrict__ p, const uint8_t* __restrict__ fix, double* __restrict__ qv, int nx,
                         int ny, size_t rows, double* __restrict__ rowsum) {
    const size_t row = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    const size_t sy = nx, sz = (size_t)nx * ny;
    const size_t base = row * (size_t)nx;
    double s = 0.0;
    for (int i = 0; i < nx; ++i) {
        const size_t q = base + i;
        double term = 0.0;
        if (fix[q]) qv[q] = 0.0;
        else {
            const double nb = p[q - 1] + p[q + 1] + p[q - sy] + p[q + sy] + p[q - sz] + p[q + sz];
            qv[q] = 6.0 * p[q] - nb;
            term = p[q] * qv[q];
        }
        s += term;
    }
    rowsum[row] = s;
}

// plane sums of the rows in j order, then the planes in k order (one block)
__global__ void k_sum_rows(const double* __restrict__ rowsum, int ny, int nz, double* __restrict__ plane,
                           double* __restrict__ out) {
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < ny; ++j) s += rowsum[(size_t)j + (size_t)ny * k];
        plane[k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < nz; ++k) s += plane[k];
        *out = s;
    }
}

// phi += alpha p, r -= alpha q, max |r|
__global__ void k_cg_update(double* __restrict__ phi, double* __restrict__ r, const double* __restrict__ p,
                            const double* __restrict__ qv, double alpha, size_t n, unsigned long long* __restrict__ rmax) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0;
    if (q < n) {
        phi[q] += alpha * p[q];
        r[q] -= alpha * qv[q];
        a = fabs(r[q]);
    }
    a = warp_max(a);
    if ((threadIdx.x & 31) == 0) max_into(rmax, a);
}

// p = z + beta p
__global__ void k_cg_dir(double* __restrict__ p, const double* __restrict__ z, double beta, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) p[q] = z[q] + beta * p[q];
}

unsigned blocks(size_t n) { return (unsigned)((n + kT - 1) / kT); }

struct Dev {
    std::vector<void*> mem;
    cudaStream_t st = nullptr;
    cudaError_t err = cudaSuccess;
    ~Dev() {
        for (void* p : mem) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, n * sizeof(T) + (n ? 0 : 16));
        if (err != cudaSuccess) return nullptr;
        mem.push_back(p);
        return static_cast<T*>(p);
    }
};

}  // namespace

extern "C" {

mq_status mq_laplace_solve_device(int32_t nx, int32_t ny, int32_t nz, const uint8_t* mask, const double* fixed,
                                  double outer_bc, double tol, int32_t device, double* phi, mq_solve_stats* stats) {
    if (nx < 3 || ny < 3 || nz < 3 || !mask || !fixed || !phi || !(tol > 0)) return MQ_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) { cudaGetLastError(); return MQ_ERR_NO_DEVICE; }
    if (cudaSetDevice(device) != cudaSuccess) return MQ_ERR_CUDA;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t n = (size_t)nx * ny * nz, rows = (size_t)ny * nz;
    const size_t sy = nx, sz = (size_t)nx * ny;
    // Dirichlet set and initial iterate exactly as the host solver builds them
    std::vector<uint8_t> fix(n);
    double maxfix = 0.0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t q = (size_t)i + sy * j + sz * k;
                const bool face = i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
                if (mask[q]) { fix[q] = 1; phi[q] = fixed[q]; maxfix = std::fmax(maxfix, std::fabs(fixed[q])); }
                else if (face) { fix[q] = 1; phi[q] = outer_bc; }
                else { fix[q] = 0; phi[q] = outer_bc; }
            }
    double scale = std::fmax(maxfix, std::fabs(outer_bc));
    if (!(scale > 0)) scale = 1.0;
    const double target = tol * scale;

    Dev D;
    if (cudaStreamCreateWithFlags(&D.st, cudaStreamNonBlocking) != cudaSuccess) return MQ_ERR_CUDA;
    const std::vector<mqlv::Dims> dims = mqlv::hierarchy(nx, ny, nz);
    std::vector<DLevel> L(dims.size());
    std::vector<uint8_t> prev = fix, cur;
    for (size_t l = 0; l < dims.size(); ++l) {
        DLevel& lv = L[l];
        lv.nx = dims[l].nx; lv.ny = dims[l].ny; lv.nz = dims[l].nz;
        if (l > 0) {
            cur.assign(lv.n(), 0);
            mqlv::coarse_fix(dims[l - 1], prev.data(), dims[l], cur.data());
            prev.swap(cur);
        }
        lv.fix = D.alloc<uint8_t>(lv.n());
        lv.u = D.alloc<double>(lv.n());
        lv.rhs = D.alloc<double>(lv.n());
        lv.r = D.alloc<double>(lv.n());
        if (D.err != cudaSuccess) return MQ_ERR_NOMEM;
        if (cudaMemcpyAsync(lv.fix, prev.data(), lv.n(), cudaMemcpyHostToDevice, D.st) != cudaSuccess) return MQ_ERR_CUDA;
        if (cudaStreamSynchronize(D.st) != cudaSuccess) return MQ_ERR_CUDA;   // prev is reused by the next level
    }
    double* dphi = D.alloc<double>(n);
    double* r = D.alloc<double>(n);
    double* p = D.alloc<double>(n);
    double* qv = D.alloc<double>(n);
    double* rowsum = D.alloc<double>(rows);
    double* plane = D.alloc<double>((size_t)nz);
    double* scal = D.alloc<double>(2);
    unsigned long long* dmax = D.alloc<unsigned long long>(1);
    if (D.err != cudaSuccess) return MQ_ERR_NOMEM;
    if (cudaMemcpyAsync(dphi, phi, n * sizeof(double), cudaMemcpyHostToDevice, D.st) != cudaSuccess) return MQ_ERR_CUDA;
    if (cudaMemsetAsync(r, 0, n * sizeof(double), D.st) != cudaSuccess) return MQ_ERR_CUDA;
    if (cudaMemsetAsync(p, 0, n * sizeof(double), D.st) != cudaSuccess) return MQ_ERR_CUDA;
    if (cudaMemsetAsync(qv, 0, n * sizeof(double), D.st) != cudaSuccess) return MQ_ERR_CUDA;
    cudaStream_t st = D.st;

    auto gs = [&](DLevel& lv, int col) {
        const size_t cnt = (size_t)((lv.nx - 1) / 2) * (lv.ny - 2) * (lv.nz - 2);
        if (cnt) k_gs<<<blocks(cnt), kT, 0, st>>>(lv.u, lv.rhs, lv.fix, lv.nx, lv.ny, lv.nz, col);
    };
    // symmetric V-cycle from u = 0 (Solver::vcycle of the host solver)
    std::function<void(size_t)> vcycle = [&](size_t l) {
        DLevel& lv = L[l];
        cudaMemsetAsync(lv.u, 0, lv.n() * sizeof(double), st);
        if (l + 1 == L.size()) {
            k_coarse<<<1, 1024, 0, st>>>(lv.u, lv.rhs, lv.fix, lv.nx, lv.ny, lv.nz, 60);
            return;
        }
        for (int s = 0; s < 2; ++s) { gs(lv, 0); gs(lv, 1); }
        k_residual<<<blocks(lv.n()), kT, 0, st>>>(lv.u, lv.rhs, lv.fix, lv.r, lv.nx, lv.ny, lv.n());
        DLevel& c = L[l + 1];
        k_restrict<<<blocks(c.n()), kT, 0, st>>>(lv.r, lv.nx, lv.ny, lv.nz, c.rhs, c.fix, c.nx, c.ny, c.nz);
        vcycle(l + 1);
        k_prolong<<<blocks(lv.n()), kT, 0, st>>>(c.u, c.nx, c.ny, lv.u, lv.fix, lv.nx, lv.ny, lv.nz);
        for (int s = 0; s < 2; ++s) { gs(lv, 1); gs(lv, 0); }
    };
    auto read_max = [&](double* out) -> bool {
        unsigned long long bits = 0;
        if (cudaMemcpyAsync(&bits, dmax, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
        if (cudaStreamSynchronize(st) != cudaSuccess) return false;
        double v;
        std::memcpy(&v, &bits, 8);
        *out = v;
        return true;
    };
    auto true_residual = [&](double* out) -> bool {
        cudaMemsetAsync(dmax, 0, 8, st);
        k_true_residual<<<blocks(n), kT, 0, st>>>(dphi, L[0].fix, r, nx, ny, n, dmax);
        return read_max(out);
    };
    auto precond = [&]() {   // L0.u = M^-1 r
        cudaMemcpyAsync(L[0].rhs, r, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        vcycle(0);
    };
    auto read_sum = [&](double* out) -> bool {
        k_sum_rows<<<1, 1024, 0, st>>>(rowsum, ny, nz, plane, scal);
        if (cudaMemcpyAsync(out, scal, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
        return cudaStreamSynchronize(st) == cudaSuccess;
    };
    auto dot_r_u = [&](double* out) -> bool {
        k_row_dot<<<blocks(rows), kT, 0, st>>>(r, L[0].u, nx, rows, rowsum);
        return read_sum(out);
    };

    double rmax = 0.0;
    if (!true_residual(&rmax)) return MQ_ERR_CUDA;
    int it = 0;
    const int max_it = 2000;
    bool converged = rmax <= target;
    while (!converged && it < max_it) {
        precond();
        cudaMemcpyAsync(p, L[0].u, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        double rz = 0.0;
        if (!dot_r_u(&rz)) return MQ_ERR_CUDA;
        int inner = 0;
        while (it < max_it) {
            k_row_sp<<<blocks(rows), kT, 0, st>>>(p, L[0].fix, qv, nx, ny, rows, rowsum);
            double pq = 0.0;
            if (!read_sum(&pq)) return MQ_ERR_CUDA;
            if (!(pq > 0)) break;
            const double alpha = rz / pq;
            cudaMemsetAsync(dmax, 0, 8, st);
            k_cg_update<<<blocks(n), kT, 0, st>>>(dphi, r, p, qv, alpha, n, dmax);
            if (!read_max(&rmax)) return MQ_ERR_CUDA;
            ++it;
            ++inner;
            if (rmax <= target || inner >= 200) break;
            precond();
            double rz_new = 0.0;
            if (!dot_r_u(&rz_new)) return MQ_ERR_CUDA;
            const double beta = rz_new / rz;
            rz = rz_new;
            k_cg_dir<<<blocks(n), kT, 0, st>>>(p, L[0].u, beta, n);
        }
        if (!true_residual(&rmax)) return MQ_ERR_CUDA;
        converged = rmax <= target;
        if (!converged && inner == 0) break;
    }
    if (cudaGetLastError() != cudaSuccess) return MQ_ERR_CUDA;
    if (cudaMemcpyAsync(phi, dphi, n * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return MQ_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MQ_ERR_CUDA;
    if (stats) {
        stats->iterations = it;
        stats->converged = converged ? 1 : 0;
        stats->final_residual = rmax / scale;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return converged ? MQ_OK : MQ_ERR_NOT_CONVERGED;
}

}  // extern "C"
