/*
 * lbm_oracle.c -- TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference CPU solver
 * (hackerbruecke/lbm). Used by tests/ as the parity checker and by bench.py's CPU arm; never by
 * the product library. Compiled with -ffp-contract=off so that every floating-point operation
 * happens in the order the reference writes it (see lbm_oracle.h for the parity pin).
 *
 * Each function cites the reference file:line it restates. Two extensions that the reference
 * does not have are marked as such: periodic axes and a per-cell inflow profile.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------------ */
/* Lattice tables: model.h:13-50 (D3Q15), 53-91 (D3Q19), 96-139 (D3Q27). The orderings must be   */
/* the reference's for population-level parity.                                                */
/* ------------------------------------------------------------------------------------------ */
static const int C15[15][3] = {
    {-1,-1,-1},{ 1,-1,-1},{ 0, 0,-1},{-1, 1,-1},{ 1, 1,-1},
    { 0,-1, 0},{-1, 0, 0},{ 0, 0, 0},{ 1, 0, 0},{ 0, 1, 0},
    {-1,-1, 1},{ 1,-1, 1},{ 0, 0, 1},{-1, 1, 1},{ 1, 1, 1}};
static const double W15[15] = {
    1.0/72, 1.0/72,  8.0/72, 1.0/72, 1.0/72,
    8.0/72, 8.0/72, 16.0/72, 8.0/72, 8.0/72,
    1.0/72, 1.0/72,  8.0/72, 1.0/72, 1.0/72};
static const int C19[19][3] = {
    { 0,-1,-1},{-1, 0,-1},{ 0, 0,-1},{ 1, 0,-1},{ 0, 1,-1},
    {-1,-1, 0},{ 0,-1, 0},{ 1,-1, 0},{-1, 0, 0},{ 0, 0, 0},
    { 1, 0, 0},{-1, 1, 0},{ 0, 1, 0},{ 1, 1, 0},{ 0,-1, 1},
    {-1, 0, 1},{ 0, 0, 1},{ 1, 0, 1},{ 0, 1, 1}};
static const double W19[19] = {
    1.0/36, 1.0/36, 2.0/36, 1.0/36, 1.0/36,
    1.0/36, 2.0/36, 1.0/36, 2.0/36, 12.0/36,
    2.0/36, 1.0/36, 2.0/36, 1.0/36, 1.0/36,
    1.0/36, 2.0/36, 1.0/36, 1.0/36};
static const int C27[27][3] = {
    {-1,-1,-1},{ 0,-1,-1},{ 1,-1,-1},{-1, 0,-1},{ 0, 0,-1},
    { 1, 0,-1},{-1, 1,-1},{ 0, 1,-1},{ 1, 1,-1},{-1,-1, 0},
    { 0,-1, 0},{ 1,-1, 0},{-1, 0, 0},{ 0, 0, 0},{ 1, 0, 0},
    {-1, 1, 0},{ 0, 1, 0},{ 1, 1, 0},{-1,-1, 1},{ 0,-1, 1},
    { 1,-1, 1},{-1, 0, 1},{ 0, 0, 1},{ 1, 0, 1},{-1, 1, 1},
    { 0, 1, 1},{ 1, 1, 1}};
static const double W27[27] = {
     1.0/216,  4.0/216,  1.0/216,  4.0/216, 16.0/216,
     4.0/216,  1.0/216,  4.0/216,  1.0/216,  4.0/216,
    16.0/216,  4.0/216, 16.0/216, 64.0/216, 16.0/216,
     4.0/216, 16.0/216,  4.0/216,  1.0/216,  4.0/216,
     1.0/216,  4.0/216, 16.0/216,  4.0/216,  1.0/216,
     4.0/216,  1.0/216};

/* lbmdefinitions.h:47: 0.57735026919l converted to double (bit pattern 0x3fe279a745904047). */
static const double CS = 0x1.279a745904047p-1;

#define QMAX 27

typedef struct {
    int type;
    double v[3];
    double rho;
    double* profile; /* extension: 3 doubles per padded cell, or NULL */
} orc_bc;

struct orc_domain {
    int Q, xl, yl, zl;
    int per[3];
    double tau;
    const int (*c)[3];
    const double* w;
    size_t ng;
    unsigned char* flag[2]; /* 0 = fluid (BGK); k >= 1 = handler k */
    double* f[2];
    int cur;                /* index of collide_field */
    int nbc;
    orc_bc bc[256];
};

static inline size_t idx(const orc_domain* d, int x, int y, int z)
{
    /* domain.hpp:60-64 */
    return (size_t)x + (size_t)(d->xl + 2) * ((size_t)y + (size_t)(d->yl + 2) * (size_t)z);
}

static inline int in_bounds(const orc_domain* d, int x, int y, int z)
{
    /* domain.hpp:66-70 */
    return x > 0 && x < d->xl + 1 && y > 0 && y < d->yl + 1 && z > 0 && z < d->zl + 1;
}

/* Extension: coordinates on periodic axes wrap into 1..l. */
static inline void wrap(const orc_domain* d, int* x, int* y, int* z)
{
    if (d->per[0]) { if (*x < 1) *x += d->xl; else if (*x > d->xl) *x -= d->xl; }
    if (d->per[1]) { if (*y < 1) *y += d->yl; else if (*y > d->yl) *y -= d->yl; }
    if (d->per[2]) { if (*z < 1) *z += d->zl; else if (*z > d->zl) *z -= d->zl; }
}

static inline int inv(const orc_domain* d, int q) { return d->Q - 1 - q; } /* model.h:36-39 */

/* model.h:41-44, 82-85, 130-133 */
static int velocity_index(const orc_domain* d, int u, int v, int w)
{
    if (d->Q == 15) return 5 * w + 2 * v + u + 7 - (w + 2) % 2 * (u + v) / 2;
    if (d->Q == 19) return w == 0 ? (6 + (v + 1) * 3 + u) : ((w + 1) * 7 + (v + 1) * 2 + u);
    return 9 * w + 3 * v + u + 13;
}

/* collision.hpp:6-14 */
static double density(const orc_domain* d, const double* cell)
{
    double rho = 0;
    for (int q = 0; q < d->Q; ++q) rho += cell[q];
    return rho;
}

/* collision.hpp:16-31 (d outer, q inner; the division by the density argument) */
static void velocity(const orc_domain* d, const double* cell, double rho, double u[3])
{
    u[0] = u[1] = u[2] = 0.0;
    for (int k = 0; k < 3; ++k)
        for (int q = 0; q < d->Q; ++q) u[k] += cell[q] * (double)d->c[q][k];
    u[0] /= rho;
    u[1] /= rho;
    u[2] /= rho;
}

/* collision.hpp:33-51, term by term as written there */
static void feq_all(const orc_domain* d, double rho, const double u[3], double* feq)
{
    for (int q = 0; q < d->Q; ++q) {
        double cu = 0.0, uu = 0.0;
        for (int k = 0; k < 3; ++k) {
            cu += (double)d->c[q][k] * u[k];
            uu += u[k] * u[k];
        }
        feq[q] = d->w[q] * rho
                 * (1 + cu / (CS * CS) + (cu) * (cu) / (2 * CS * CS * CS * CS)
                    - uu / (2 * CS * CS));
    }
}

/* collision.hpp:60-70 */
static void bgk(const orc_domain* d, double* cell)
{
    double u[3], feq[QMAX];
    const double rho = density(d, cell);
    velocity(d, cell, rho, u);
    feq_all(d, rho, u, feq);
    for (int q = 0; q < d->Q; ++q) cell[q] -= (cell[q] - feq[q]) / d->tau;
}

static int is_fluid_at(const orc_domain* d, const unsigned char* fl, int x, int y, int z)
{
    return fl[idx(d, x, y, z)] == 0;
}

/* The non-fluid handlers, boundary.hpp:14-214. `f` is the current collide_field. */
static void boundary_collide(const orc_domain* d, const unsigned char* fl, double* f,
                             int x, int y, int z, const orc_bc* bc)
{
    const int Q = d->Q;
    double* cell = f + idx(d, x, y, z) * Q;
    for (int q = 0; q < Q; ++q) {
        const int dx = d->c[q][0], dy = d->c[q][1], dz = d->c[q][2];
        int nx = x + dx, ny = y + dy, nz = z + dz;
        wrap(d, &nx, &ny, &nz);
        if (!(in_bounds(d, nx, ny, nz) && is_fluid_at(d, fl, nx, ny, nz))) continue;
        const double* nb = f + idx(d, nx, ny, nz) * Q;
        switch (bc->type) {
        case ORC_NOSLIP: /* boundary.hpp:14-31 */
            cell[q] = nb[inv(d, q)];
            break;
        case ORC_MOVINGWALL: { /* boundary.hpp:43-68 */
            const double rho = density(d, nb);
            double cu = 0;
            for (int k = 0; k < 3; ++k) cu += (double)d->c[q][k] * bc->v[k];
            const double finv = nb[inv(d, q)];
            cell[q] = finv + 2.0 * d->w[q] * rho * cu / (CS * CS);
            break;
        }
        case ORC_FREESLIP: { /* boundary.hpp:79-115, fallback order x, y, z, yz, xz, xy */
            int cx[6][3] = {{x + dx, y, z}, {x, y + dy, z}, {x, y, z + dz},
                            {x, y + dy, z + dz}, {x + dx, y, z + dz}, {x + dx, y + dy, z}};
            const int mir[6][3] = {{-dx, dy, dz}, {dx, -dy, dz}, {dx, dy, -dz},
                                   {dx, -dy, -dz}, {-dx, dy, -dz}, {-dx, -dy, dz}};
            for (int k = 0; k < 6; ++k) {
                wrap(d, &cx[k][0], &cx[k][1], &cx[k][2]);
                if (is_fluid_at(d, fl, cx[k][0], cx[k][1], cx[k][2])) {
                    const double* src = f + idx(d, cx[k][0], cx[k][1], cx[k][2]) * Q;
                    cell[q] = src[velocity_index(d, mir[k][0], mir[k][1], mir[k][2])];
                    break;
                }
            }
            break;
        }
        case ORC_OUTFLOW:   /* boundary.hpp:128-150 */
        case ORC_PRESSURE: { /* boundary.hpp:194-214: same formula with rho-in */
            double u[3], feq[QMAX];
            velocity(d, nb, bc->rho, u);
            feq_all(d, bc->rho, u, feq);
            cell[q] = feq[q] + feq[inv(d, q)] - nb[inv(d, q)];
            break;
        }
        case ORC_INFLOW: { /* boundary.hpp:164-181 (+ per-cell profile extension) */
            double feq[QMAX];
            const double* v = bc->v;
            if (bc->profile) v = bc->profile + 3 * idx(d, x, y, z);
            feq_all(d, bc->rho, v, feq);
            cell[q] = feq[q];
            break;
        }
        default:
            break;
        }
    }
}

orc_domain* orc_create(int q, int xl, int yl, int zl, double tau)
{
    if (xl < 1 || yl < 1 || zl < 1) return NULL;
    orc_domain* d = (orc_domain*)calloc(1, sizeof(orc_domain));
    if (!d) return NULL;
    d->Q = q;
    d->xl = xl; d->yl = yl; d->zl = zl;
    d->tau = tau;
    if (q == 15) { d->c = C15; d->w = W15; }
    else if (q == 19) { d->c = C19; d->w = W19; }
    else if (q == 27) { d->c = C27; d->w = W27; }
    else { free(d); return NULL; }
    d->ng = (size_t)(xl + 2) * (size_t)(yl + 2) * (size_t)(zl + 2);
    for (int k = 0; k < 2; ++k) {
        d->flag[k] = (unsigned char*)calloc(d->ng, 1);
        d->f[k] = (double*)malloc(d->ng * (size_t)q * sizeof(double));
        if (!d->flag[k] || !d->f[k]) { orc_destroy(d); return NULL; }
        /* cell.hpp:8-15: every cell starts at the weights */
        for (size_t i = 0; i < d->ng; ++i) memcpy(d->f[k] + i * q, d->w, q * sizeof(double));
    }
    d->cur = 0;
    return d;
}

void orc_destroy(orc_domain* d)
{
    if (!d) return;
    for (int k = 0; k < 2; ++k) { free(d->flag[k]); free(d->f[k]); }
    for (int b = 0; b < d->nbc; ++b) free(d->bc[b].profile);
    free(d);
}

int orc_add_boundary(orc_domain* d, int type, const double params[4])
{
    if (type < ORC_NOSLIP || type > ORC_PRESSURE || d->nbc >= 255) return -1;
    orc_bc* b = &d->bc[d->nbc];
    b->type = type;
    b->v[0] = params[0]; b->v[1] = params[1]; b->v[2] = params[2];
    b->rho = params[3];
    b->profile = NULL;
    return ++d->nbc;
}

int orc_set_boundary_box(orc_domain* d, int handler, const int64_t e[6])
{
    if (handler < 1 || handler > d->nbc) return -1;
    /* domain.hpp:180-181 asserts */
    if (!(e[1] >= e[0] && e[3] >= e[2] && e[5] >= e[4])) return -1;
    if (!(e[1] < d->xl + 2 && e[3] < d->yl + 2 && e[5] < d->zl + 2) || e[0] < 0 || e[2] < 0 || e[4] < 0)
        return -1;
    for (int64_t z = e[4]; z <= e[5]; ++z)
        for (int64_t y = e[2]; y <= e[3]; ++y)
            for (int64_t x = e[0]; x <= e[1]; ++x) {
                const size_t i = idx(d, (int)x, (int)y, (int)z);
                d->flag[0][i] = (unsigned char)handler;
                d->flag[1][i] = (unsigned char)handler;
            }
    return 0;
}

int orc_set_solid(orc_domain* d, const unsigned char* mask, int mode)
{
    const double zero[4] = {0, 0, 0, 1};
    const int h = orc_add_boundary(d, ORC_NOSLIP, zero);
    if (h < 0) return -1;
    size_t m = 0;
    for (int z = 1; z <= d->zl; ++z)
        for (int y = 1; y <= d->yl; ++y)
            for (int x = 1; x <= d->xl; ++x, ++m) {
                if (!mask[m]) continue;
                const size_t i = idx(d, x, y, z);
                d->flag[d->cur][i] = (unsigned char)h;
                if (mode == 0) d->flag[1 - d->cur][i] = (unsigned char)h;
            }
    return h;
}

int orc_set_periodic(orc_domain* d, int px, int py, int pz)
{
    d->per[0] = px != 0; d->per[1] = py != 0; d->per[2] = pz != 0;
    return 0;
}

int orc_set_inflow_profile(orc_domain* d, int handler, const double* u_cells)
{
    if (handler < 1 || handler > d->nbc || d->bc[handler - 1].type != ORC_INFLOW) return -1;
    orc_bc* b = &d->bc[handler - 1];
    if (!b->profile) b->profile = (double*)malloc(3 * d->ng * sizeof(double));
    if (!b->profile) return -1;
    memcpy(b->profile, u_cells, 3 * d->ng * sizeof(double));
    return 0;
}

int orc_set_populations(orc_domain* d, const double* f)
{
    memcpy(d->f[d->cur], f, d->ng * (size_t)d->Q * sizeof(double));
    return 0;
}

int orc_get_populations(const orc_domain* d, double* f)
{
    memcpy(f, d->f[d->cur], d->ng * (size_t)d->Q * sizeof(double));
    return 0;
}

static int axis_active(const orc_domain* d, int x, int y, int z)
{
    /* ghost cells of a periodic axis are never read; skip them in the collide sweep */
    if (d->per[0] && (x == 0 || x == d->xl + 1)) return 0;
    if (d->per[1] && (y == 0 || y == d->yl + 1)) return 0;
    if (d->per[2] && (z == 0 || z == d->zl + 1)) return 0;
    return 1;
}

/* domain.hpp:115-141 (pull stream into stream_field, interior fluid cells only) */
static void stream(orc_domain* d)
{
    const int Q = d->Q;
    const double* src = d->f[d->cur];
    double* dst = d->f[1 - d->cur];
    const unsigned char* fl = d->flag[d->cur];
    const int xl = d->xl, yl = d->yl, zl = d->zl;
#pragma omp parallel for collapse(3) schedule(static)
    for (int z = 1; z <= zl; ++z)
        for (int y = 1; y <= yl; ++y)
            for (int x = 1; x <= xl; ++x) {
                const size_t i = idx(d, x, y, z);
                if (fl[i] != 0) continue;
                for (int q = 0; q < Q; ++q) {
                    int sx = x - d->c[q][0], sy = y - d->c[q][1], sz = z - d->c[q][2];
                    wrap(d, &sx, &sy, &sz);
                    dst[i * Q + q] = src[idx(d, sx, sy, sz) * Q + q];
                }
            }
}

/* domain.hpp:143-166: phase A (fluid cells, incl. ghost layer) then phase B (non-fluid) */
static void collide(orc_domain* d)
{
    const int Q = d->Q;
    double* f = d->f[d->cur];
    const unsigned char* fl = d->flag[d->cur];
    const int xl = d->xl, yl = d->yl, zl = d->zl;
#pragma omp parallel for collapse(3) schedule(static)
    for (int z = 0; z < zl + 2; ++z)
        for (int y = 0; y < yl + 2; ++y)
            for (int x = 0; x < xl + 2; ++x) {
                const size_t i = idx(d, x, y, z);
                if (fl[i] == 0 && axis_active(d, x, y, z)) bgk(d, f + i * Q);
            }
#pragma omp parallel for collapse(3) schedule(static)
    for (int z = 0; z < zl + 2; ++z)
        for (int y = 0; y < yl + 2; ++y)
            for (int x = 0; x < xl + 2; ++x) {
                const size_t i = idx(d, x, y, z);
                if (fl[i] != 0) boundary_collide(d, fl, f, x, y, z, &d->bc[fl[i] - 1]);
            }
}

int orc_step(orc_domain* d, int nsteps, int threads, double* seconds)
{
    if (threads > 0) omp_set_num_threads(threads);
    double total = 0.0;
    for (int t = 0; t < nsteps; ++t) {
        const double t0 = omp_get_wtime();
        stream(d);
        d->cur = 1 - d->cur; /* domain.hpp:168-172 */
        collide(d);
        total += omp_get_wtime() - t0;
    }
    if (seconds) *seconds = total;
    return 0;
}

int orc_moments(const orc_domain* d, double* rho, double* u)
{
    const int Q = d->Q;
    const double* f = d->f[d->cur];
    size_t m = 0;
    for (int z = 1; z <= d->zl; ++z)
        for (int y = 1; y <= d->yl; ++y)
            for (int x = 1; x <= d->xl; ++x, ++m) {
                const double* cell = f + idx(d, x, y, z) * Q;
                const double r = density(d, cell);
                double v[3];
                velocity(d, cell, r, v);
                if (rho) rho[m] = r;
                if (u) { u[3 * m] = v[0]; u[3 * m + 1] = v[1]; u[3 * m + 2] = v[2]; }
            }
    return 0;
}

double orc_cs(void) { return CS; }
