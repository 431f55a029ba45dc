// Multigrid level geometry shared by the host and device Laplace solvers: vertex-centred
// coarsening n -> n/2 + 1, and the Dirichlet mask of a coarse level (its boundary faces, fine
// nodes that are fixed, and coarse nodes beyond the fine grid).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace mqlv {

struct Dims { int nx, ny, nz; };

inline size_t count(const Dims& d) { return (size_t)d.nx * d.ny * d.nz; }

// level dims below the finest (empty when the grid is already coarse)
inline std::vector<Dims> hierarchy(int nx, int ny, int nz) {
    std::vector<Dims> L{{nx, ny, nz}};
    for (;;) {
        const Dims f = L.back();
        const int cx = f.nx / 2 + 1, cy = f.ny / 2 + 1, cz = f.nz / 2 + 1;
        if (f.nx < 5 || f.ny < 5 || f.nz < 5 || cx < 3 || cy < 3 || cz < 3) break;
        L.push_back({cx, cy, cz});
    }
    return L;
}

inline void coarse_fix(const Dims& f, const uint8_t* ffix, const Dims& c, uint8_t* cfix) {
    for (int K = 0; K < c.nz; ++K)
        for (int J = 0; J < c.ny; ++J)
            for (int I = 0; I < c.nx; ++I) {
                bool fx = I == 0 || J == 0 || K == 0 || I == c.nx - 1 || J == c.ny - 1 || K == c.nz - 1;
                if (!fx) {
                    const int i = 2 * I, j = 2 * J, k = 2 * K;
                    fx = (i >= f.nx || j >= f.ny || k >= f.nz)
                             ? true
                             : ffix[(size_t)i + (size_t)f.nx * ((size_t)j + (size_t)f.ny * k)] != 0;
                }
                cfix[(size_t)I + (size_t)c.nx * ((size_t)J + (size_t)c.ny * K)] = fx ? 1 : 0;
            }
}

}  // namespace mqlv
