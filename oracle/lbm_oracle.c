/*
 * C restatement of the pylabolt fluidLB CPU kernels -- TEST INFRASTRUCTURE.
 *
 * Used by the tests as the FP64 oracle for cases too large for the NumPy
 * restatement, and by bench.py as the timed CPU baseline (FP64, or the FP32
 * build for single-precision workloads).  It is never linked into or called
 * by the product library.
 *
 * It keeps the reference's structure: padded AoS populations [node][9], node
 * index x*(Ny+2)+y, one parallel sweep per reference kernel (OpenMP over nodes,
 * the counterpart of numba prange), and the reference's per-node floating
 * point operation order.  Build with -ffp-contract=off so no multiply-add is
 * fused: results are then bit-identical to the reference kernels run as
 * Python (checked against tests/golden).  Kernels restated:
 *   density   pylabolt/parallel/cpu/compute_fields_kernels.py:5-28
 *   force     pylabolt/parallel/cpu/force_field_kernels.py:5-25
 *   velocity  pylabolt/parallel/cpu/compute_fields_kernels.py:31-65
 *   BGK       pylabolt/parallel/cpu/collision_kernels.py:5-153
 *   wrap      pylabolt/parallel/gpu/MPI_kernels.py:51-99
 *   stream    pylabolt/parallel/cpu/streaming_kernels.py:5-47
 *   BCs       pylabolt/parallel/cpu/fluid_boundary_kernels.py:5-62,100-152
 *   residue   pylabolt/parallel/cpu/compute_residues_kernels.py:6-73
 * MRT and zero_gradient follow the project's own definitions (no reference
 * kernel exists); see oracle/lbm_np.py.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

/* Type of the fields and of the per-node arithmetic: double for the FP64
 * oracle; float (-DOR_REAL=float) for the "precision": "single" case, whose
 * state.fields arrays are float32 (pylabolt/base/control.py:36-40,
 * pylabolt/base/fields.py:64-92), timed as the CPU baseline of
 * single-precision workloads.  As in the reference's Numba kernels on float32
 * arrays, double-precision constants promote the expressions they appear in;
 * the residue sums stay in double. */
#ifndef OR_REAL
#define OR_REAL double
#endif
typedef OR_REAL real;

static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int INVD[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

typedef struct {
    int64_t nxp, nyp;          /* padded extents */
    int32_t collision;         /* 0 BGK, 1 MRT */
    int32_t forcing;           /* 0 None, 1 guo_linear, 2 guo_second_order */
    int32_t x_periodic, y_periodic;
    int32_t periodic_selfcopy; /* 1: single-rank CPU self copy, 0: true wrap */
    int32_t pad_;
    double omega, inv_cs_2, inv_cs_4, eps;
    double gravity[2];
    double w[9];
    double mrt_s[9];           /* diagonal of S */
    double m[81], minv[81];    /* MRT transform and its inverse (row-major) */
} OrParams;

typedef struct {
    int32_t type;      /* 0 bounce_back, 1 fixed_velocity, 2 fixed_pressure, 3 zero_gradient */
    int32_t normal[2];
    int32_t out_list[3], inv_list[3];
    int32_t pad_;
    double value[2];
    int64_t node_begin, node_end;   /* range in the concatenated node array */
} OrElement;

static void compute_moments(const OrParams *p, const int64_t *idx, int64_t n,
                            const real *pop_new, real *density,
                            real *velocity, real *force,
                            const real *body_force) {
    int64_t t;
#pragma omp parallel for schedule(static)
    for (t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        const real *f = pop_new + 9 * ind;
        real s = 0.;
        for (int k = 0; k < 9; ++k) s += f[k];
        density[ind] = s;
    }
#pragma omp parallel for schedule(static)
    for (t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        if (body_force) {
            force[2 * ind] = body_force[2 * ind];
            force[2 * ind + 1] = body_force[2 * ind + 1];
        } else {
            real r = density[ind];
            force[2 * ind] = r * p->gravity[0];
            force[2 * ind + 1] = r * p->gravity[1];
        }
    }
#pragma omp parallel for schedule(static)
    for (t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        const real *f = pop_new + 9 * ind;
        real sx = 0., sy = 0.;
        for (int k = 0; k < 9; ++k) {
            sx += (real)CX[k] * f[k];
            sy += (real)CY[k] * f[k];
        }
        real inv_density = 1 / (density[ind] + p->eps);
        velocity[2 * ind] = sx * inv_density + 0.5 * force[2 * ind] * inv_density;
        velocity[2 * ind + 1] = sy * inv_density + 0.5 * force[2 * ind + 1] * inv_density;
    }
}

static inline real feq_k(const OrParams *p, int k, real rho, real ux,
                           real uy, real u2) {
    real cu = (real)CX[k] * ux + (real)CY[k] * uy;
    return p->w[k] * rho *
           (1 + p->inv_cs_2 * cu + 0.5 * p->inv_cs_4 * cu * cu - 0.5 * p->inv_cs_2 * u2);
}

static inline real guo_k(const OrParams *p, int k, real ux, real uy,
                           real fx, real fy) {
    if (p->forcing == 1)
        return p->w[k] * ((real)CX[k] * fx + (real)CY[k] * fy) * p->inv_cs_2;
    real cu = (real)CX[k] * ux + (real)CY[k] * uy;
    real const_x = ((real)CX[k] - ux) * p->inv_cs_2 + cu * (real)CX[k] * p->inv_cs_4;
    real const_y = ((real)CY[k] - uy) * p->inv_cs_2 + cu * (real)CY[k] * p->inv_cs_4;
    return p->w[k] * (const_x * fx + const_y * fy);
}

static void collide(const OrParams *p, const int64_t *idx, int64_t n,
                    const real *density, const real *velocity,
                    const real *force, real *pop, const real *pop_new) {
    int64_t t;
    const real omega = p->omega;
#pragma omp parallel for schedule(static)
    for (t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        real rho = density[ind];
        real ux = velocity[2 * ind], uy = velocity[2 * ind + 1];
        real fx = force[2 * ind], fy = force[2 * ind + 1];
        real u2 = ux * ux + uy * uy;
        const real *fn = pop_new + 9 * ind;
        real *fo = pop + 9 * ind;
        if (p->collision == 0) {
            for (int k = 0; k < 9; ++k) {
                real pop_eq = feq_k(p, k, rho, ux, uy, u2);
                if (p->forcing == 0)
                    fo[k] = (1 - omega) * fn[k] + omega * pop_eq;
                else
                    fo[k] = (1 - omega) * fn[k] + omega * pop_eq +
                            (1 - 0.5 * omega) * guo_k(p, k, ux, uy, fx, fy);
            }
        } else {
            real m[9], meq[9], mf[9], fe[9], fb[9], ms[9];
            for (int k = 0; k < 9; ++k) {
                fe[k] = feq_k(p, k, rho, ux, uy, u2);
                fb[k] = p->forcing ? guo_k(p, k, ux, uy, fx, fy) : 0.0;
            }
            for (int a = 0; a < 9; ++a) {
                real s0 = 0, s1 = 0, s2 = 0;
                for (int k = 0; k < 9; ++k) {
                    s0 += p->m[9 * a + k] * fn[k];
                    s1 += p->m[9 * a + k] * fe[k];
                    s2 += p->m[9 * a + k] * fb[k];
                }
                m[a] = s0; meq[a] = s1; mf[a] = s2;
            }
            for (int a = 0; a < 9; ++a)
                ms[a] = m[a] - p->mrt_s[a] * (m[a] - meq[a]) + (1 - 0.5 * p->mrt_s[a]) * mf[a];
            for (int k = 0; k < 9; ++k) {
                real s = 0;
                for (int a = 0; a < 9; ++a) s += p->minv[9 * k + a] * ms[a];
                fo[k] = s;
            }
        }
    }
}

static void halo(const OrParams *p, real *pop) {
    const int64_t nxp = p->nxp, nyp = p->nyp;
    if (p->x_periodic) {
        int64_t sl = p->periodic_selfcopy ? 1 : nxp - 2;
        int64_t sr = p->periodic_selfcopy ? nxp - 2 : 1;
        for (int64_t y = 0; y < nyp; ++y)
            for (int k = 0; k < 9; ++k) {
                pop[9 * (0 * nyp + y) + k] = pop[9 * (sl * nyp + y) + k];
                pop[9 * ((nxp - 1) * nyp + y) + k] = pop[9 * (sr * nyp + y) + k];
            }
    }
    if (p->y_periodic) {
        int64_t sb = p->periodic_selfcopy ? 1 : nyp - 2;
        int64_t st = p->periodic_selfcopy ? nyp - 2 : 1;
        for (int64_t x = 0; x < nxp; ++x)
            for (int k = 0; k < 9; ++k) {
                pop[9 * (x * nyp + 0) + k] = pop[9 * (x * nyp + sb) + k];
                pop[9 * (x * nyp + nyp - 1) + k] = pop[9 * (x * nyp + st) + k];
            }
    }
}

static void stream(const OrParams *p, const int64_t *idx, int64_t n,
                   const uint8_t *solid, const real *density,
                   const real *velocity, const real *pop, real *pop_new) {
    int64_t t;
    const int64_t nyp = p->nyp;
#pragma omp parallel for schedule(static)
    for (t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        real density_local = density[ind];
        pop_new[9 * ind] = pop[9 * ind];
        for (int k = 1; k < 9; ++k) {
            int64_t nb = ind - CX[k] * nyp - CY[k];
            if (!solid[nb]) {
                pop_new[9 * ind + k] = pop[9 * nb + k];
            } else {
                int ki = INVD[k];
                real temp = 2 * p->w[ki] * density_local * p->inv_cs_2 *
                              ((real)CX[ki] * velocity[2 * nb] +
                               (real)CY[ki] * velocity[2 * nb + 1]);
                pop_new[9 * ind + k] = pop[9 * ind + ki] - temp;
            }
        }
    }
}

static void boundaries(const OrParams *p, const OrElement *el, int32_t nel,
                       const int64_t *nodes, const uint8_t *solid,
                       const real *density, const real *velocity,
                       const real *pop, real *pop_new) {
    const int64_t nyp = p->nyp, nxp = p->nxp;
    for (int32_t e = 0; e < nel; ++e) {
        const OrElement *E = el + e;
        int64_t b;
#pragma omp parallel for schedule(static)
        for (b = E->node_begin; b < E->node_end; ++b) {
            int64_t ind = nodes[b];
            if (solid[ind]) continue;
            if (E->type == 0) {
                for (int k = 0; k < 3; ++k)
                    pop_new[9 * ind + E->inv_list[k]] = pop[9 * ind + E->out_list[k]];
            } else if (E->type == 1) {
                real density_local = density[ind];
                for (int k = 0; k < 3; ++k) {
                    int o = E->out_list[k], i = E->inv_list[k];
                    real temp = 2 * p->w[o] * density_local * p->inv_cs_2 *
                                  ((real)CX[o] * E->value[0] + (real)CY[o] * E->value[1]);
                    pop_new[9 * ind + i] = pop[9 * ind + o] - temp;
                }
            } else if (E->type == 2) {
                int64_t nrm = ind + E->normal[0] * nyp + E->normal[1];
                real ux = velocity[2 * ind], uy = velocity[2 * ind + 1];
                real uex = ux + 0.5 * (ux - velocity[2 * nrm]);
                real uey = uy + 0.5 * (uy - velocity[2 * nrm + 1]);
                real u2 = uex * uex + uey * uey;
                for (int k = 0; k < 3; ++k) {
                    int o = E->out_list[k], i = E->inv_list[k];
                    real cu = (real)CX[o] * uex + (real)CY[o] * uey;
                    real temp = 2 * p->w[o] * E->value[0] *
                                  (1 + 0.5 * p->inv_cs_4 * cu * cu - 0.5 * p->inv_cs_2 * u2);
                    pop_new[9 * ind + i] = -pop[9 * ind + o] + temp;
                }
            } else if (E->type == 3) {
                int64_t bx = ind / nyp - 1, by = ind % nyp - 1;
                int64_t nx = nxp - 2, ny = nyp - 2;
                int64_t fb = ind + E->normal[0] * nyp + E->normal[1];
                for (int k = 0; k < 3; ++k) {
                    int i = E->inv_list[k];
                    int64_t x = bx + E->normal[0] - CX[i];
                    int64_t y = by + E->normal[1] - CY[i];
                    if (p->x_periodic) x = ((x % nx) + nx) % nx;
                    if (p->y_periodic) y = ((y % ny) + ny) % ny;
                    int64_t src = fb;
                    if (x >= 0 && x < nx && y >= 0 && y < ny) {
                        int64_t s = (x + 1) * nyp + (y + 1);
                        if (!solid[s]) src = s;
                    }
                    pop_new[9 * ind + i] = pop[9 * src + i];
                }
            }
        }
    }
}

/* Initial equilibrium -- pylabolt/parallel/cpu/equilibrium_kernels.py:38-78 */
void or_initialize(const OrParams *p, const int64_t *idx, int64_t n,
                   const real *density, const real *velocity, real *pop,
                   real *pop_new) {
    int64_t t;
#pragma omp parallel for schedule(static)
    for (t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        real ux = velocity[2 * ind], uy = velocity[2 * ind + 1];
        real u2 = ux * ux + uy * uy;
        for (int k = 0; k < 9; ++k) {
            real v = feq_k(p, k, density[ind], ux, uy, u2);
            pop[9 * ind + k] = v;
            pop_new[9 * ind + k] = v;
        }
    }
}

/* nsteps of Solver.single_time_step (pylabolt/solvers/fluidLB.py:206-253). */
void or_run(const OrParams *p, const int64_t *idx, int64_t n,
            const uint8_t *solid, real *density, real *velocity,
            real *force, real *pop, real *pop_new,
            const real *body_force, const OrElement *el, int32_t nel,
            const int64_t *nodes, int64_t nsteps) {
    for (int64_t s = 0; s < nsteps; ++s) {
        compute_moments(p, idx, n, pop_new, density, velocity, force, body_force);
        collide(p, idx, n, density, velocity, force, pop, pop_new);
        halo(p, pop);
        stream(p, idx, n, solid, density, velocity, pop, pop_new);
        boundaries(p, el, nel, nodes, solid, density, velocity, pop, pop_new);
    }
}

/* Residue sums in node order; updates the old fields.
 * out = {num_rho, den_rho, num_ux, den_ux, num_uy, den_uy}. */
void or_residue(const int64_t *idx, int64_t n, const real *density,
                const real *velocity, real *density_old,
                real *velocity_old, double *out) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t t = 0; t < n; ++t) {
        int64_t ind = idx[t];
        double d = (double)density[ind] - (double)density_old[ind];
        s[0] += d * d;
        s[1] += (double)density_old[ind] * (double)density_old[ind];
        density_old[ind] = density[ind];
        for (int c = 0; c < 2; ++c) {
            double o = velocity_old[2 * ind + c];
            double v = (double)velocity[2 * ind + c] - o;
            s[2 + 2 * c] += v * v;
            s[3 + 2 * c] += o * o;
            velocity_old[2 * ind + c] = velocity[2 * ind + c];
        }
    }
    memcpy(out, s, sizeof(s));
}
