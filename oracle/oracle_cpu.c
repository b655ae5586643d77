/*
 * oracle_cpu.c -- CPU restatement of TopOpt.jl's matrix-free SIMP path in C
 * (TEST INFRASTRUCTURE AND CPU BASELINE ONLY; never linked into the product).
 *
 * It follows the reference algorithm step by step so that its run time stands
 * for the reference's Julia CPU path (Julia is not available on these
 * machines).  Paths relative to the TopOpt.jl project root:
 *   orc_matvec   src/FEA/matrix_free_operator.jl:66-105 -- per element
 *                xes_e = rho_e * bcmatrix(Ke_e) * x_e with one Ke copy per element
 *                (ElementFEAInfo stores one Symmetric SMatrix per cell,
 *                src/TopOptProblems/elementinfo.jl:75-100), then each free dof
 *                gathers its (cell, local) entries through dof_cells; fixed dofs
 *                get meandiag * x.
 *   orc_pcg      src/FEA/solvers_api.jl:177-220 -> IterativeSolvers cg! with a
 *                diagonal (Jacobi) preconditioner: tol = max(rtol*||r0||, abstol).
 *   orc_compliance  src/Functions/compute_element_energy.jl:18-38.
 *   orc_filter_J / orc_filter_JT  node-based filter J = M2 M1
 *                (src/CheqFilters/density_filter.jl:49-108, CheqFilters.jl:66-118)
 *                with the per-node valence weight of the reference's BFS.
 *   orc_oc       published OC update (88-line code), no reference counterpart.
 * OpenMP parallelises the element and dof loops; the reference itself is
 * single-threaded (1 thread reproduces it).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int dim, nel[3], nn[3], ndpc;
    int64_t nnodes, ncells, ndofs;
    const int32_t* cell_dofs; /* ncells * ndpc */
    double* Kes;              /* ncells * ndpc * ndpc (per-element copies) */
    const uint8_t* fixed;     /* per dof */
    double meandiag, xmin, p;
    double* rho;              /* per cell */
    int64_t* dc_off;          /* dof_cells CSR */
    int32_t* dc_cell;
    int8_t* dc_loc;
    double* xes;              /* ncells * ndpc */
    double* diag;             /* Jacobi diagonal per dof */
} orc_op;

static double penal(double x, double p) { return pow(x, p); }

orc_op* orc_create(int dim, const int32_t* nel, const int32_t* cell_dofs, const double* Ke, const uint8_t* fixed,
                   double xmin, double p) {
    orc_op* o = (orc_op*)calloc(1, sizeof(orc_op));
    o->dim = dim;
    o->nnodes = 1;
    o->ncells = 1;
    for (int d = 0; d < 3; ++d) {
        o->nel[d] = d < dim ? nel[d] : 1;
        o->nn[d] = d < dim ? nel[d] + 1 : 1;
        if (d < dim) {
            o->nnodes *= o->nn[d];
            o->ncells *= o->nel[d];
        }
    }
    o->ndofs = o->nnodes * dim;
    o->ndpc = (1 << dim) * dim;
    o->cell_dofs = cell_dofs;
    o->fixed = fixed;
    o->xmin = xmin;
    o->p = p;
    const int nd = o->ndpc;
    o->Kes = (double*)malloc(sizeof(double) * o->ncells * nd * nd);
    double tr = 0;
    for (int i = 0; i < nd; ++i) tr += Ke[i * nd + i];
    o->meandiag = tr * (double)o->ncells; /* solvers_api.jl:526-527 */
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) memcpy(o->Kes + e * nd * nd, Ke, sizeof(double) * nd * nd);
    o->rho = (double*)malloc(sizeof(double) * o->ncells);
    o->xes = (double*)malloc(sizeof(double) * o->ncells * nd);
    o->diag = (double*)malloc(sizeof(double) * o->ndofs);
    /* dof_cells in cell order (metadata.jl:64-76) */
    o->dc_off = (int64_t*)calloc(o->ndofs + 1, sizeof(int64_t));
    for (int64_t e = 0; e < o->ncells; ++e)
        for (int l = 0; l < nd; ++l) o->dc_off[cell_dofs[e * nd + l] + 1]++;
    for (int64_t d = 0; d < o->ndofs; ++d) o->dc_off[d + 1] += o->dc_off[d];
    o->dc_cell = (int32_t*)malloc(sizeof(int32_t) * o->ncells * nd);
    o->dc_loc = (int8_t*)malloc(o->ncells * nd);
    int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * o->ndofs);
    memcpy(pos, o->dc_off, sizeof(int64_t) * o->ndofs);
    for (int64_t e = 0; e < o->ncells; ++e)
        for (int l = 0; l < nd; ++l) {
            const int32_t d = cell_dofs[e * nd + l];
            o->dc_cell[pos[d]] = (int32_t)e;
            o->dc_loc[pos[d]] = (int8_t)l;
            pos[d]++;
        }
    free(pos);
    return o;
}

void orc_destroy(orc_op* o) {
    if (!o) return;
    free(o->Kes);
    free(o->rho);
    free(o->xes);
    free(o->diag);
    free(o->dc_off);
    free(o->dc_cell);
    free(o->dc_loc);
    free(o);
}

void orc_set_threads(int n) { omp_set_num_threads(n); }
int orc_max_threads(void) { return omp_get_max_threads(); }

void orc_set_vars(orc_op* o, const double* vars) {
    const int nd = o->ndpc;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) o->rho[e] = penal(vars[e], o->p) * (1 - o->xmin) + o->xmin;
    /* Jacobi diagonal of the masked operator */
    for (int64_t d = 0; d < o->ndofs; ++d) o->diag[d] = 0.0;
    for (int64_t e = 0; e < o->ncells; ++e)
        for (int l = 0; l < nd; ++l) o->diag[o->cell_dofs[e * nd + l]] += o->rho[e] * o->Kes[e * nd * nd + l * nd + l];
    for (int64_t d = 0; d < o->ndofs; ++d)
        if (o->fixed[d]) o->diag[d] = o->meandiag;
}

void orc_matvec(orc_op* o, const double* x, double* y) {
    const int nd = o->ndpc;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) {
        double xe[24], m[24];
        const int32_t* cd = o->cell_dofs + e * nd;
        for (int j = 0; j < nd; ++j) {
            m[j] = o->fixed[cd[j]] ? 0.0 : 1.0;
            xe[j] = x[cd[j]] * m[j];
        }
        const double* K = o->Kes + e * nd * nd;
        double* out = o->xes + e * nd;
        for (int i = 0; i < nd; ++i) {
            double s = 0.0;
            for (int j = 0; j < nd; ++j) s += K[i * nd + j] * xe[j];
            out[i] = o->rho[e] * m[i] * s;
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < o->ndofs; ++d) {
        if (o->fixed[d]) {
            y[d] = o->meandiag * x[d];
            continue;
        }
        double s = 0.0;
        for (int64_t k = o->dc_off[d]; k < o->dc_off[d + 1]; ++k) s += o->xes[(int64_t)o->dc_cell[k] * nd + o->dc_loc[k]];
        y[d] = s;
    }
}

static double dot(const double* a, const double* b, int64_t n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* Jacobi PCG from x = 0 (initially_zero).  Runs at most maxit iterations;
 * returns the iteration count, *res = final recurrence residual norm. */
int orc_pcg(orc_op* o, const double* b, double* x, double rtol, double abstol, int maxit, double* res) {
    const int64_t n = o->ndofs;
    double* r = (double*)malloc(sizeof(double) * n);
    double* u = (double*)calloc(n, sizeof(double));
    double* c = (double*)malloc(sizeof(double) * n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        x[i] = 0.0;
        r[i] = o->fixed[i] ? 0.0 : b[i];
    }
    double rn = sqrt(dot(r, r, n));
    const double tol = fmax(rtol * rn, abstol);
    double rho = 1.0;
    int it = 0;
    while (it < maxit && rn > tol) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) c[i] = r[i] / o->diag[i];
        const double rho_prev = rho;
        rho = dot(c, r, n);
        const double beta = rho / rho_prev;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) u[i] = c[i] + beta * u[i];
        orc_matvec(o, u, c);
        const double alpha = rho / dot(u, c, n);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * u[i];
            r[i] -= alpha * c[i];
        }
        rn = sqrt(dot(r, r, n));
        ++it;
    }
    if (res) *res = rn;
    free(r);
    free(u);
    free(c);
    return it;
}

double orc_compliance(orc_op* o, const double* u, const double* vars, double* grad) {
    const int nd = o->ndpc;
    double c = 0.0;
#pragma omp parallel for reduction(+ : c) schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) {
        const int32_t* cd = o->cell_dofs + e * nd;
        const double* K = o->Kes + e * nd * nd;
        double ce = 0.0;
        for (int w = 0; w < nd; ++w)
            for (int v = 0; v < nd; ++v) ce += u[cd[v]] * K[v * nd + w] * u[cd[w]];
        const double x = vars[e];
        const double rho = penal(x, o->p) * (1 - o->xmin) + o->xmin;
        const double drho = (1 - o->xmin) * o->p * (o->p == 0 ? 0.0 : pow(x, o->p - 1));
        grad[e] = -drho * ce;
        c += rho * ce;
    }
    return c;
}

/* ---- node-based filter with a stencil of node offsets (dx,dy,dz) and weights ---- */
static int valence(const orc_op* o, int ix, int iy, int iz) {
    int v = (ix > 0 && ix < o->nel[0] ? 2 : 1) * (iy > 0 && iy < o->nel[1] ? 2 : 1);
    if (o->dim == 3) v *= (iz > 0 && iz < o->nel[2] ? 2 : 1);
    return v;
}

static void node_avg(const orc_op* o, const double* xe, double* nodal) {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < o->nnodes; ++n) {
        const int ix = (int)(n % o->nn[0]), iy = (int)((n / o->nn[0]) % o->nn[1]), iz = (int)(n / ((int64_t)o->nn[0] * o->nn[1]));
        double s = 0.0;
        int cnt = 0;
        for (int bz = 0; bz < (o->dim == 3 ? 2 : 1); ++bz)
            for (int by = 0; by < 2; ++by)
                for (int bx = 0; bx < 2; ++bx) {
                    const int cx = ix - 1 + bx, cy = iy - 1 + by, cz = o->dim == 3 ? iz - 1 + bz : 0;
                    if (cx >= 0 && cx < o->nel[0] && cy >= 0 && cy < o->nel[1] && cz >= 0 && cz < o->nel[2]) {
                        s += xe[cx + (int64_t)o->nel[0] * (cy + (int64_t)o->nel[1] * cz)];
                        ++cnt;
                    }
                }
        nodal[n] = cnt ? s / cnt : 0.0;
    }
}

void orc_filter_J(const orc_op* o, const int* soff, const double* sw, int S, const double* x, double* y, double* nodal) {
    node_avg(o, x, nodal);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) {
        const int ex = (int)(e % o->nel[0]), ey = (int)((e / o->nel[0]) % o->nel[1]), ez = (int)(e / ((int64_t)o->nel[0] * o->nel[1]));
        double s = 0.0, W = 0.0;
        for (int k = 0; k < S; ++k) {
            const int ix = ex + soff[3 * k], iy = ey + soff[3 * k + 1], iz = ez + soff[3 * k + 2];
            if (ix >= 0 && ix < o->nn[0] && iy >= 0 && iy < o->nn[1] && iz >= 0 && iz < o->nn[2]) {
                const double w = sw[k] * valence(o, ix, iy, iz);
                s += w * nodal[ix + (int64_t)o->nn[0] * (iy + (int64_t)o->nn[1] * iz)];
                W += w;
            }
        }
        y[e] = W > 0 ? s / W : x[e];
    }
}

void orc_filter_JT(const orc_op* o, const int* soff, const double* sw, int S, const double* d, double* y, double* nodal,
                   double* invW) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) {
        const int ex = (int)(e % o->nel[0]), ey = (int)((e / o->nel[0]) % o->nel[1]), ez = (int)(e / ((int64_t)o->nel[0] * o->nel[1]));
        double W = 0.0;
        for (int k = 0; k < S; ++k) {
            const int ix = ex + soff[3 * k], iy = ey + soff[3 * k + 1], iz = ez + soff[3 * k + 2];
            if (ix >= 0 && ix < o->nn[0] && iy >= 0 && iy < o->nn[1] && iz >= 0 && iz < o->nn[2])
                W += sw[k] * valence(o, ix, iy, iz);
        }
        invW[e] = W > 0 ? 1.0 / W : 0.0;
    }
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < o->nnodes; ++n) {
        const int ix = (int)(n % o->nn[0]), iy = (int)((n / o->nn[0]) % o->nn[1]), iz = (int)(n / ((int64_t)o->nn[0] * o->nn[1]));
        double s = 0.0;
        for (int k = 0; k < S; ++k) {
            const int ex = ix - soff[3 * k], ey = iy - soff[3 * k + 1], ez = iz - soff[3 * k + 2];
            if (ex >= 0 && ex < o->nel[0] && ey >= 0 && ey < o->nel[1] && ez >= 0 && ez < o->nel[2]) {
                const int64_t e = ex + (int64_t)o->nel[0] * (ey + (int64_t)o->nel[1] * ez);
                s += sw[k] * invW[e] * d[e];
            }
        }
        nodal[n] = s * valence(o, ix, iy, iz);
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < o->ncells; ++e) {
        const int ex = (int)(e % o->nel[0]), ey = (int)((e / o->nel[0]) % o->nel[1]), ez = (int)(e / ((int64_t)o->nel[0] * o->nel[1]));
        double s = 0.0;
        for (int j = 0; j < (1 << o->dim); ++j) {
            const int ix = ex + (j & 1), iy = ey + ((j >> 1) & 1), iz = ez + ((j >> 2) & 1);
            s += nodal[ix + (int64_t)o->nn[0] * (iy + (int64_t)o->nn[1] * iz)] / valence(o, ix, iy, iz);
        }
        y[e] = s;
    }
}

/* OC bisection (88-line code): returns lambda; xnew written, *change = max|xnew - x| */
double orc_oc(int64_t n, const double* x, const double* dc, const double* dv, const double* w, double volfrac,
              double move, double* xnew, double* change) {
    double* B = (double*)malloc(sizeof(double) * n);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; ++e) B[e] = x[e] * sqrt(fmax(0.0, -dc[e]) / dv[e]);
    double l1 = 0.0, l2 = 1e9;
    while ((l2 - l1) / (l1 + l2) > 1e-3) {
        const double lmid = 0.5 * (l2 + l1), s = 1.0 / sqrt(lmid);
        double vol = 0.0;
#pragma omp parallel for reduction(+ : vol) schedule(static)
        for (int64_t e = 0; e < n; ++e) {
            const double xn = fmin(fmin(1.0, x[e] + move), fmax(fmax(0.0, x[e] - move), B[e] * s));
            vol += w[e] * xn;
        }
        if (vol > volfrac)
            l1 = lmid;
        else
            l2 = lmid;
    }
    const double lmid = 0.5 * (l2 + l1), s = 1.0 / sqrt(lmid);
    double ch = 0.0;
#pragma omp parallel for reduction(max : ch) schedule(static)
    for (int64_t e = 0; e < n; ++e) {
        xnew[e] = fmin(fmin(1.0, x[e] + move), fmax(fmax(0.0, x[e] - move), B[e] * s));
        ch = fmax(ch, fabs(xnew[e] - x[e]));
    }
    *change = ch;
    free(B);
    return lmid;
}
