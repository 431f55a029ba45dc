// Parametric geometry of the 486-quadrupole trap cube with its nine exit ports (host and
// device).  Restates trapsim Geometry (simulation/trapsim/src/geometry.rs:12-205): lattice
// of posts on the cube faces, wall planes with clearance holes, port rods continuing outside
// the wall, end caps, port apertures.  All lengths in mm; evaluated in IEEE double without FMA
// contraction so host and device classify a point identically.
#pragma once
#include <math.h>
#include <stdint.h>

#include "mq_tandem.h"

#if defined(__CUDACC__)
#define MQC_HD __host__ __device__ __forceinline__
#else
#define MQC_HD inline
#endif

namespace mqc {

constexpr int ID_FREE = 0, ID_POST = 1, ID_PLANE = 2, ID_ENT = 3, ID_EXT = 4;   // geometry.rs:12-16

MQC_HD double c0(const mq_cube_geom& g) { return g.t_pcb + g.gap + g.d / 2.0; }
MQC_HD double size(const mq_cube_geom& g) { return 2.0 * c0(g) + (double)(g.n - 1) * g.pitch; }
MQC_HD double lat(const mq_cube_geom& g, int i) { return c0(g) + g.pitch * (double)i; }
MQC_HD double post_top_depth(const mq_cube_geom& g) { return g.t_pcb + g.gap + g.height; }

// post on lattice point idx belongs to face axis a (priority z > y > x), geometry.rs:81-86
MQC_HD bool post_valid(const mq_cube_geom& g, int a, const int idx[3]) {
    if (idx[a] != 0 && idx[a] != g.n - 1) return false;
    for (int a2 = a + 1; a2 < 3; ++a2)
        if (idx[a2] == 0 || idx[a2] == g.n - 1) return false;
    return true;
}

// exit port of index i (nine ports in a 3x3 array), geometry.rs:114-117
MQC_HD void port(const mq_cube_geom& g, int index, int out[4]) {   // axis, side, cell0, cell1
    out[0] = g.ext_axis; out[1] = g.ext_side;
    if (!g.array) { out[2] = g.ext_cell[0]; out[3] = g.ext_cell[1]; return; }
    out[2] = 2 + 2 * (index % 3);
    out[3] = 2 + 2 * (index / 3);
}

// port axis centre (b, c axes and their coordinates), geometry.rs:109-113
MQC_HD void port_axis_xy(const mq_cube_geom& g, const int p[4], int* b, int* c, double* xb, double* xc) {
    const int a = p[0];
    *b = (a + 1) % 3;
    *c = (a + 2) % 3;
    *xb = 0.5 * (lat(g, p[2]) + lat(g, p[2] + 1));
    *xc = 0.5 * (lat(g, p[3]) + lat(g, p[3] + 1));
}

MQC_HD double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// v.round() clamped to [0, hi] and cast to an index the way Rust's saturating `as usize` does (NaN -> 0)
MQC_HD int round_idx(double v, int hi) {
    const double r = round(v);
    if (!(r > 0.0)) return 0;
    return r < (double)hi ? (int)r : hi;
}

// nearest of the nine mouths, geometry.rs:118-125
MQC_HD int nearest_port(const mq_cube_geom& g, double x, double y) {
    if (!g.array) return 0;
    const double first = (lat(g, 2) + lat(g, 3)) / 2.0;
    return round_idx((x - first) / (2.0 * g.pitch), 2) + 3 * round_idx((y - first) / (2.0 * g.pitch), 2);
}

MQC_HD void port_posts(const mq_cube_geom& g, const int p[4], int out[4][3]) {   // geometry.rs:96-108
    const int a = p[0], b = (a + 1) % 3, c = (a + 2) % 3;
    int m = 0;
    for (int db = 0; db < 2; ++db)
        for (int dc = 0; dc < 2; ++dc) {
            out[m][a] = p[1] == 0 ? 0 : g.n - 1;
            out[m][b] = p[2] + db;
            out[m][c] = p[3] + dc;
            ++m;
        }
}

MQC_HD double dist2d(double u, double v) { return sqrt(u * u + v * v); }

// classify a point (mm), electrode growth gr: returns id, sets the RF sign (geometry.rs:136-205)
MQC_HD int classify(const mq_cube_geom& g, const double p[3], double gr, int* sign_out) {
    const double l = size(g);
    const int n = g.n;
    const double half_d = g.d / 2.0;
    int found_id = ID_FREE, found_sign = 0;
    bool plane = false;
    const bool inside = p[0] >= -1e-12 && p[0] <= l + 1e-12 && p[1] >= -1e-12 && p[1] <= l + 1e-12 && p[2] >= -1e-12 &&
                        p[2] <= l + 1e-12;
    const int ent[4] = {g.ent_axis, g.ent_side, g.ent_cell[0], g.ent_cell[1]};
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        for (int side = 0; side < 2; ++side) {
            const double u = side == 0 ? p[a] : l - p[a];
            int pid = 0;       // port id on this face: 0 none, ID_ENT or ID_EXT
            int ps[4] = {0, 0, 0, 0};
            if (g.ent_axis == a && g.ent_side == side) { pid = ID_ENT; for (int q = 0; q < 4; ++q) ps[q] = ent[q]; }
            else if (g.ext_axis == a && g.ext_side == side) { pid = ID_EXT; port(g, nearest_port(g, p[b], p[c]), ps); }
            // outside the cube: only port rods (and the end cap)
            if (u < 0.0 || (pid != 0 && u < 0.0 + 1e-12)) {
                if (pid != 0) {
                    if (u <= -(g.l_ext + g.cap_gap)) {
                        int bb, cc;
                        double cb, ccx;
                        port_axis_xy(g, ps, &bb, &cc, &cb, &ccx);
                        if (dist2d(p[b] - cb, p[c] - ccx) < g.cap_r) { *sign_out = 0; return pid; }
                    }
                    if (u >= -(g.l_ext + gr)) {
                        int pp[4][3];
                        port_posts(g, ps, pp);
                        for (int m = 0; m < 4; ++m) {
                            const double dd = dist2d(p[b] - lat(g, pp[m][b]), p[c] - lat(g, pp[m][c]));
                            if (dd < half_d + gr) {
                                *sign_out = ((pp[m][0] + pp[m][1] + pp[m][2]) % 2 == 0) ? 1 : -1;
                                return pid;
                            }
                        }
                    }
                }
                continue;
            }
            if (!inside || u > post_top_depth(g) + gr) continue;
            // nearest lattice post in-plane
            const int ib = round_idx((p[b] - c0(g)) / g.pitch, n - 1), ic = round_idx((p[c] - c0(g)) / g.pitch, n - 1);
            int idx[3];
            idx[a] = side == 0 ? 0 : n - 1;
            idx[b] = ib;
            idx[c] = ic;
            const bool valid = post_valid(g, a, idx);
            const double dd = dist2d(p[b] - lat(g, ib), p[c] - lat(g, ic));
            const int sign = ((idx[0] + idx[1] + idx[2]) % 2 == 0) ? 1 : -1;
            int port_post = 0;
            bool aperture = false;
            if (pid != 0) {
                if (valid) {
                    int pp[4][3];
                    port_posts(g, ps, pp);
                    for (int m = 0; m < 4; ++m)
                        if (pp[m][0] == idx[0] && pp[m][1] == idx[1] && pp[m][2] == idx[2]) port_post = pid;
                }
                int bb, cc;
                double cb, ccx;
                port_axis_xy(g, ps, &bb, &cc, &cb, &ccx);
                if (dist2d(p[b] - cb, p[c] - ccx) < g.ap_r - gr) aperture = true;
            }
            if (port_post != 0)   // rod: full radius from the wall to the post top
                if (u <= post_top_depth(g) + gr && dd < half_d + gr) { *sign_out = sign; return port_post; }
            if (u <= g.t_pcb + gr) {   // wall plane
                const double hole_r = port_post != 0 ? half_d + g.rod_clear_extra : g.clear_r;
                const bool in_hole = aperture || (valid && dd < hole_r - gr);
                if (!in_hole) plane = true;
            }
            if (valid && port_post == 0) {   // stem + post
                if (u <= g.t_pcb + g.gap + gr && dd < g.stem_r + gr) { found_id = ID_POST; found_sign = sign; }
                if (u >= g.t_pcb + g.gap - gr && u <= post_top_depth(g) + gr && dd < half_d + gr) { found_id = ID_POST; found_sign = sign; }
            }
        }
    }
    if (found_id != ID_FREE) { *sign_out = found_sign; return found_id; }
    *sign_out = 0;
    return plane ? ID_PLANE : ID_FREE;
}

}  // namespace mqc
