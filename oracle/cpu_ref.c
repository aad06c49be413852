/*
 * CPU oracle for the phonomena elastic FDTD time-stepping solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the GPU library never
 * links it, and only tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.
 *
 * Two restatements live here:
 *
 *  (1) ora_f64_*: the reference's displacement-stress leapfrog, FP64, with the
 *      exact IEEE operation order of the reference's NumPy expressions, so that
 *      its output is bit-identical to phonomena's own solver.  It keeps the
 *      reference structure: six stress arrays recomputed from u every step,
 *      then the displacement update, the traction-free z=0 rows, the absorbing
 *      faces in the reference order, and the copy-rotation.
 *        source overwrite      simulation/base_solver.py:251
 *        update_T              simulation/base_solver.py:329-372
 *        apply_T_tfbc          simulation/base_solver.py:408-433
 *        update_u              simulation/base_solver.py:441-463
 *        apply_u_tfbc          simulation/base_solver.py:495-516 (surface_mode
 *                              0 keeps the precedence of :516, 1 corrects it)
 *        apply_u_abc           simulation/base_solver.py:525-554
 *        time_step             simulation/base_solver.py:561-571
 *      Generalisations: any number of material ids (a uint8 id per node and a
 *      13-entry table per id instead of the per-node 6x6 C and P), a rigid-wall
 *      option for the four absorbing faces, and a full-wall source option.
 *
 *  (2) ora_f32k_*: the FP32 velocity-form scheme with Kahan-compensated
 *      displacement integration that the GPU FP32 kernel implements, restated
 *      with the same per-value operation sequence (explicit fmaf, no other
 *      contraction) so that GPU and CPU agree bit for bit.  In exact
 *      arithmetic it equals (1) when v(-1/2) = 0.
 *
 * Build with -ffp-contract=off (no implicit FMA) and without -ffast-math.
 * Arrays use the reference shapes, C order (x slowest):
 *   ux (nx-1, ny, nz)   uy (nx, ny-1, nz)   uz (nx, ny, nz-1)
 *   T1..T3 (nx, ny, nz) T4 (nx, ny-1, nz-1) T5 (nx-1, ny, nz-1) T6 (nx-1, ny-1, nz)
 * nx, ny, nz are NODE counts (Grid.x.size etc.), all >= 3.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORA_NTAB 13 /* C00 C01 C02 C10 C11 C12 C20 C21 C22 C33 C44 C55 P */

typedef struct {
    int nx, ny, nz;
    const double *fdx, *fdy, *fdz; /* n-1 full spacings (SI) */
    const double *sdx, *sdy, *sdz; /* n-2 staggered spacings (SI) */
    const uint8_t *mat;            /* nx*ny*nz node material ids */
    const double *table;           /* nmat * 13 */
    int nmat;
    double dt;
    const double *src; /* source sample per global step */
    int nsrc;
    int surface_mode; /* 0 reference precedence, 1 corrected */
    int bc;           /* 0 absorbing faces (reference), 1 rigid faces */
    int source_mode;  /* 0 line uz[0,:,0] (reference), 1 wall uz[0,:,:] */
} ora_problem;

/* index helpers: a (d0, d1, d2) array */
#define I3(d1, d2, i, j, k) ((((size_t)(i)) * (size_t)(d1) + (size_t)(j)) * (size_t)(d2) + (size_t)(k))

static int set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int ora_max_threads(void) { return set_threads(0); }

/* ABC coefficients in the reference order: clx[-1], ctx[-1], cty[0], cly[0],
 * cty[-1], cly[-1], ctz[-1], clz[-1] (simulation/base_solver.py:525-537),
 * taken from the material at node (0,0,0). */
void ora_abc_coeffs(const ora_problem *p, double out[8]) {
    const double *t = p->table + (size_t)p->mat[0] * ORA_NTAB;
    double vl = sqrt(t[0] / t[12]);
    double vt = sqrt(t[9] / t[12]);
    double vld = vl * p->dt, vtd = vt * p->dt;
    int nx = p->nx, ny = p->ny, nz = p->nz;
    out[0] = (vld - p->sdx[nx - 3]) / (vld + p->sdx[nx - 3]); /* clx[-1] */
    out[1] = (vtd - p->fdx[nx - 2]) / (vtd + p->fdx[nx - 2]); /* ctx[-1] */
    out[2] = (vtd - p->fdy[0]) / (vtd + p->fdy[0]);           /* cty[0] */
    out[3] = (vld - p->sdy[0]) / (vld + p->sdy[0]);           /* cly[0] */
    out[4] = (vtd - p->fdy[ny - 2]) / (vtd + p->fdy[ny - 2]); /* cty[-1] */
    out[5] = (vld - p->sdy[ny - 3]) / (vld + p->sdy[ny - 3]); /* cly[-1] */
    out[6] = (vtd - p->fdz[nz - 2]) / (vtd + p->fdz[nz - 2]); /* ctz[-1] */
    out[7] = (vld - p->sdz[nz - 3]) / (vld + p->sdz[nz - 3]); /* clz[-1] */
}

/* ------------------------------------------------------------------------ */
/* (1) FP64 reference leapfrog                                               */
/* ------------------------------------------------------------------------ */

typedef struct {
    double *ux, *uy, *uz;             /* u (current) */
    double *ux_old, *uy_old, *uz_old; /* u at the previous step */
    double *ux_new, *uy_new, *uz_new; /* last written u_new (kept across steps) */
} ora_f64_state;

typedef struct {
    double *T1, *T2, *T3, *T4, *T5, *T6;
} ora_f64_stress;

static void f64_stress(const ora_problem *p, const ora_f64_state *s, ora_f64_stress *T) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const double *ux = s->ux, *uy = s->uy, *uz = s->uz;
    const double *tab = p->table;
    const uint8_t *mat = p->mat;
    /* T1..T3 interior [1:-1,1:-1,1:-1] (base_solver.py:329-351) */
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 1; k <= nz - 2; k++) {
                const double *c = tab + (size_t)mat[I3(ny, nz, i, j, k)] * ORA_NTAB;
                double dux = ux[I3(ny, nz, i, j, k)] - ux[I3(ny, nz, i - 1, j, k)];
                double duy = uy[I3(ny - 1, nz, i, j, k)] - uy[I3(ny - 1, nz, i, j - 1, k)];
                double duz = uz[I3(ny, nz - 1, i, j, k)] - uz[I3(ny, nz - 1, i, j, k - 1)];
                double a = p->sdx[i - 1], b = p->sdy[j - 1], d = p->sdz[k - 1];
                size_t o = I3(ny, nz, i, j, k);
                T->T1[o] = ((c[0] * dux) / a + (c[1] * duy) / b) + (c[2] * duz) / d;
                T->T2[o] = ((c[3] * dux) / a + (c[4] * duy) / b) + (c[5] * duz) / d;
                T->T3[o] = ((c[6] * dux) / a + (c[7] * duy) / b) + (c[8] * duz) / d;
            }
    /* T4 [1:-1,:,:] (:353-358) */
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                const double *c = tab + (size_t)mat[I3(ny, nz, i, j + 1, k + 1)] * ORA_NTAB;
                double a = (uy[I3(ny - 1, nz, i, j, k + 1)] - uy[I3(ny - 1, nz, i, j, k)]) / p->fdz[k];
                double b = (uz[I3(ny, nz - 1, i, j + 1, k)] - uz[I3(ny, nz - 1, i, j, k)]) / p->fdy[j];
                T->T4[I3(ny - 1, nz - 1, i, j, k)] = c[9] * (a + b);
            }
    /* T5 [:,1:-1,:] (:360-365) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                const double *c = tab + (size_t)mat[I3(ny, nz, i + 1, j, k + 1)] * ORA_NTAB;
                double a = (ux[I3(ny, nz, i, j, k + 1)] - ux[I3(ny, nz, i, j, k)]) / p->fdz[k];
                double b = (uz[I3(ny, nz - 1, i + 1, j, k)] - uz[I3(ny, nz - 1, i, j, k)]) / p->fdx[i];
                T->T5[I3(ny, nz - 1, i, j, k)] = c[10] * (a + b);
            }
    /* T6 [:,:,1:-1] (:367-372) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++)
            for (int k = 1; k <= nz - 2; k++) {
                const double *c = tab + (size_t)mat[I3(ny, nz, i + 1, j + 1, k)] * ORA_NTAB;
                double a = (ux[I3(ny, nz, i, j + 1, k)] - ux[I3(ny, nz, i, j, k)]) / p->fdy[j];
                double b = (uy[I3(ny - 1, nz, i + 1, j, k)] - uy[I3(ny - 1, nz, i, j, k)]) / p->fdx[i];
                T->T6[I3(ny - 1, nz, i, j, k)] = c[11] * (a + b);
            }
    /* traction-free z=0 rows (:408-433).  The reference divides by the first
     * element of each spacing array ([0,:,:] etc. broadcast as a scalar), and
     * T4/T5/T6 use the spacing arrays listed there; both are kept. */
    const double sdx0 = p->sdx[0], sdy0 = p->sdy[0], sdz0 = p->sdz[0];
    const double fdx0 = p->fdx[0], fdy0 = p->fdy[0], fdz0 = p->fdz[0];
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++) {
            const double *c = tab + (size_t)mat[I3(ny, nz, i, j, 0)] * ORA_NTAB;
            double dux = ux[I3(ny, nz, i, j, 0)] - ux[I3(ny, nz, i - 1, j, 0)];
            double duy = uy[I3(ny - 1, nz, i, j, 0)] - uy[I3(ny - 1, nz, i, j - 1, 0)];
            double duz = uz[I3(ny, nz - 1, i, j, 0)] - 0.0;
            size_t o = I3(ny, nz, i, j, 0);
            T->T1[o] = ((c[0] * dux) / sdx0 + (c[1] * duy) / sdy0) + (c[2] * duz) / sdz0;
            T->T2[o] = ((c[3] * dux) / sdx0 + (c[4] * duy) / sdy0) + (c[5] * duz) / sdz0;
            T->T3[o] = 0.0;
        }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++) {
            const double *c = tab + (size_t)mat[I3(ny, nz, i, j + 1, 0)] * ORA_NTAB;
            double a = (uy[I3(ny - 1, nz, i, j, 1)] - uy[I3(ny - 1, nz, i, j, 0)]) / fdy0;
            double b = (uz[I3(ny, nz - 1, i, j + 1, 0)] - uz[I3(ny, nz - 1, i, j, 0)]) / fdz0;
            T->T4[I3(ny - 1, nz - 1, i, j, 0)] = c[9] * (a + b);
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++) {
            const double *c = tab + (size_t)mat[I3(ny, nz, i + 1, j, 0)] * ORA_NTAB;
            double a = (ux[I3(ny, nz, i, j, 1)] - ux[I3(ny, nz, i, j, 0)]) / fdx0;
            double b = (uz[I3(ny, nz - 1, i + 1, j, 0)] - uz[I3(ny, nz - 1, i, j, 0)]) / fdz0;
            T->T5[I3(ny, nz - 1, i, j, 0)] = c[10] * (a + b);
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++) {
            const double *c = tab + (size_t)mat[I3(ny, nz, i + 1, j + 1, 0)] * ORA_NTAB;
            double a = (ux[I3(ny, nz, i, j + 1, 0)] - ux[I3(ny, nz, i, j, 0)]) / fdx0;
            double b = (uy[I3(ny - 1, nz, i + 1, j, 0)] - uy[I3(ny - 1, nz, i, j, 0)]) / fdz0;
            T->T6[I3(ny - 1, nz, i, j, 0)] = c[11] * (a + b);
        }
}

static void f64_update(const ora_problem *p, const ora_f64_state *s, const ora_f64_stress *T) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const double *tab = p->table;
    const uint8_t *mat = p->mat;
    const double dt2 = p->dt * p->dt;
    /* ux_new[:,1:-1,1:-1] (:441-447) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 1; k <= nz - 2; k++) {
                double P = tab[(size_t)mat[I3(ny, nz, i + 1, j, k)] * ORA_NTAB + 12];
                double a = (T->T1[I3(ny, nz, i + 1, j, k)] - T->T1[I3(ny, nz, i, j, k)]) / p->fdx[i];
                double b = (T->T6[I3(ny - 1, nz, i, j, k)] - T->T6[I3(ny - 1, nz, i, j - 1, k)]) / p->sdy[j - 1];
                double c = (T->T5[I3(ny, nz - 1, i, j, k)] - T->T5[I3(ny, nz - 1, i, j, k - 1)]) / p->sdz[k - 1];
                size_t o = I3(ny, nz, i, j, k);
                s->ux_new[o] = (2.0 * s->ux[o] - s->ux_old[o]) + (dt2 / P) * ((a + b) + c);
            }
    /* uy_new[1:-1,:,1:-1] (:449-455) */
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++)
            for (int k = 1; k <= nz - 2; k++) {
                double P = tab[(size_t)mat[I3(ny, nz, i, j + 1, k)] * ORA_NTAB + 12];
                double a = (T->T6[I3(ny - 1, nz, i, j, k)] - T->T6[I3(ny - 1, nz, i - 1, j, k)]) / p->sdx[i - 1];
                double b = (T->T2[I3(ny, nz, i, j + 1, k)] - T->T2[I3(ny, nz, i, j, k)]) / p->fdy[j];
                double c = (T->T4[I3(ny - 1, nz - 1, i, j, k)] - T->T4[I3(ny - 1, nz - 1, i, j, k - 1)]) / p->sdz[k - 1];
                size_t o = I3(ny - 1, nz, i, j, k);
                s->uy_new[o] = (2.0 * s->uy[o] - s->uy_old[o]) + (dt2 / P) * ((a + b) + c);
            }
    /* uz_new[1:-1,1:-1,:] (:457-463) */
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                double P = tab[(size_t)mat[I3(ny, nz, i, j, k + 1)] * ORA_NTAB + 12];
                double a = (T->T5[I3(ny, nz - 1, i, j, k)] - T->T5[I3(ny, nz - 1, i - 1, j, k)]) / p->sdx[i - 1];
                double b = (T->T4[I3(ny - 1, nz - 1, i, j, k)] - T->T4[I3(ny - 1, nz - 1, i, j - 1, k)]) / p->sdy[j - 1];
                double c = (T->T3[I3(ny, nz, i, j, k + 1)] - T->T3[I3(ny, nz, i, j, k)]) / p->fdz[k];
                size_t o = I3(ny, nz - 1, i, j, k);
                s->uz_new[o] = (2.0 * s->uz[o] - s->uz_old[o]) + (dt2 / P) * ((a + b) + c);
            }
    /* traction-free z=0 rows of u_new (:495-516) */
    const double sdx0 = p->sdx[0], sdy0 = p->sdy[0], sdz0 = p->sdz[0];
    const double fdx0 = p->fdx[0], fdy0 = p->fdy[0], fdz0 = p->fdz[0];
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++) {
            double P = tab[(size_t)mat[I3(ny, nz, i + 1, j, 0)] * ORA_NTAB + 12];
            double a = (T->T1[I3(ny, nz, i + 1, j, 0)] - T->T1[I3(ny, nz, i, j, 0)]) / fdx0;
            double b = (T->T6[I3(ny - 1, nz, i, j, 0)] - T->T6[I3(ny - 1, nz, i, j - 1, 0)]) / sdy0;
            double c = (T->T5[I3(ny, nz - 1, i, j, 0)] - 0.0) / sdz0;
            size_t o = I3(ny, nz, i, j, 0);
            s->ux_new[o] = (2.0 * s->ux[o] - s->ux_old[o]) + (dt2 / P) * ((a + b) + c);
        }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++) {
            double P = tab[(size_t)mat[I3(ny, nz, i, j + 1, 0)] * ORA_NTAB + 12];
            double a = (T->T6[I3(ny - 1, nz, i, j, 0)] - T->T6[I3(ny - 1, nz, i - 1, j, 0)]) / sdx0;
            double b = (T->T2[I3(ny, nz, i, j + 1, 0)] - T->T2[I3(ny, nz, i, j, 0)]) / fdy0;
            double c = (T->T4[I3(ny - 1, nz - 1, i, j, 0)] - 0.0) / sdz0;
            size_t o = I3(ny - 1, nz, i, j, 0);
            s->uy_new[o] = (2.0 * s->uy[o] - s->uy_old[o]) + (dt2 / P) * ((a + b) + c);
        }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++) {
            /* density at z index 0, not 1: P[1:-1,1:-1,0] at :513 */
            double P = tab[(size_t)mat[I3(ny, nz, i, j, 0)] * ORA_NTAB + 12];
            double a = (T->T5[I3(ny, nz - 1, i, j, 0)] - T->T5[I3(ny, nz - 1, i - 1, j, 0)]) / sdx0;
            double b = (T->T4[I3(ny - 1, nz - 1, i, j, 0)] - T->T4[I3(ny - 1, nz - 1, i, j - 1, 0)]) / sdy0;
            double t31 = T->T3[I3(ny, nz, i, j, 1)], t30 = T->T3[I3(ny, nz, i, j, 0)];
            double sum;
            if (p->surface_mode == 0)
                sum = ((a + b) + t31) - t30 / fdz0; /* precedence of :516 */
            else
                sum = (a + b) + (t31 - t30) / fdz0;
            size_t o = I3(ny, nz - 1, i, j, 0);
            s->uz_new[o] = (2.0 * s->uz[o] - s->uz_old[o]) + (dt2 / P) * sum;
        }
}

/* Absorbing faces in the reference order x=N, y=0, y=N, z=N (:540-554); each
 * face reads the plane next to it as it stands after the earlier faces. */
static void f64_faces(const ora_problem *p, const ora_f64_state *s) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    double *ux = s->ux, *uy = s->uy, *uz = s->uz;
    double *xn = s->ux_new, *yn = s->uy_new, *zn = s->uz_new;
    double c[8];
    int rigid = p->bc == 1;
    if (!rigid) ora_abc_coeffs(p, c);
    else memset(c, 0, sizeof c);
#define ABC(dst, nbr_new, nbr_old, self_old, coef) \
    (dst) = rigid ? 0.0 : ((nbr_old) + (coef) * ((nbr_new) - (self_old)))
    /* x = N */
    for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz; k++)
            ABC(xn[I3(ny, nz, nx - 2, j, k)], xn[I3(ny, nz, nx - 3, j, k)], ux[I3(ny, nz, nx - 3, j, k)],
                ux[I3(ny, nz, nx - 2, j, k)], c[0]);
    for (int j = 0; j < ny - 1; j++)
        for (int k = 0; k < nz; k++)
            ABC(yn[I3(ny - 1, nz, nx - 1, j, k)], yn[I3(ny - 1, nz, nx - 2, j, k)], uy[I3(ny - 1, nz, nx - 2, j, k)],
                uy[I3(ny - 1, nz, nx - 1, j, k)], c[1]);
    for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz - 1; k++)
            ABC(zn[I3(ny, nz - 1, nx - 1, j, k)], zn[I3(ny, nz - 1, nx - 2, j, k)], uz[I3(ny, nz - 1, nx - 2, j, k)],
                uz[I3(ny, nz - 1, nx - 1, j, k)], c[1]);
    /* y = 0 */
    for (int i = 0; i < nx - 1; i++)
        for (int k = 0; k < nz; k++)
            ABC(xn[I3(ny, nz, i, 0, k)], xn[I3(ny, nz, i, 1, k)], ux[I3(ny, nz, i, 1, k)], ux[I3(ny, nz, i, 0, k)],
                c[2]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz; k++)
            ABC(yn[I3(ny - 1, nz, i, 0, k)], yn[I3(ny - 1, nz, i, 1, k)], uy[I3(ny - 1, nz, i, 1, k)],
                uy[I3(ny - 1, nz, i, 0, k)], c[3]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz - 1; k++)
            ABC(zn[I3(ny, nz - 1, i, 0, k)], zn[I3(ny, nz - 1, i, 1, k)], uz[I3(ny, nz - 1, i, 1, k)],
                uz[I3(ny, nz - 1, i, 0, k)], c[2]);
    /* y = N */
    for (int i = 0; i < nx - 1; i++)
        for (int k = 0; k < nz; k++)
            ABC(xn[I3(ny, nz, i, ny - 1, k)], xn[I3(ny, nz, i, ny - 2, k)], ux[I3(ny, nz, i, ny - 2, k)],
                ux[I3(ny, nz, i, ny - 1, k)], c[4]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz; k++)
            ABC(yn[I3(ny - 1, nz, i, ny - 2, k)], yn[I3(ny - 1, nz, i, ny - 3, k)], uy[I3(ny - 1, nz, i, ny - 3, k)],
                uy[I3(ny - 1, nz, i, ny - 2, k)], c[5]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz - 1; k++)
            ABC(zn[I3(ny, nz - 1, i, ny - 1, k)], zn[I3(ny, nz - 1, i, ny - 2, k)], uz[I3(ny, nz - 1, i, ny - 2, k)],
                uz[I3(ny, nz - 1, i, ny - 1, k)], c[4]);
    /* z = N */
    for (int i = 0; i < nx - 1; i++)
        for (int j = 0; j < ny; j++)
            ABC(xn[I3(ny, nz, i, j, nz - 1)], xn[I3(ny, nz, i, j, nz - 2)], ux[I3(ny, nz, i, j, nz - 2)],
                ux[I3(ny, nz, i, j, nz - 1)], c[6]);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny - 1; j++)
            ABC(yn[I3(ny - 1, nz, i, j, nz - 1)], yn[I3(ny - 1, nz, i, j, nz - 2)], uy[I3(ny - 1, nz, i, j, nz - 2)],
                uy[I3(ny - 1, nz, i, j, nz - 1)], c[6]);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            ABC(zn[I3(ny, nz - 1, i, j, nz - 2)], zn[I3(ny, nz - 1, i, j, nz - 3)], uz[I3(ny, nz - 1, i, j, nz - 3)],
                uz[I3(ny, nz - 1, i, j, nz - 2)], c[7]);
#undef ABC
}

static void apply_source_f64(const ora_problem *p, double *uz, int tt) {
    const int ny = p->ny, nz = p->nz;
    double s = p->src[tt];
    if (p->source_mode == 0) {
        for (int j = 0; j < ny; j++) uz[I3(ny, nz - 1, 0, j, 0)] = s;
    } else {
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz - 1; k++) uz[I3(ny, nz - 1, 0, j, k)] = s;
    }
}

static int check_problem(const ora_problem *p) {
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) return -1;
    if (!p->fdx || !p->fdy || !p->fdz || !p->sdx || !p->sdy || !p->sdz || !p->mat || !p->table) return -2;
    if (p->nmat < 1 || p->nmat > 256) return -3;
    size_t n = (size_t)p->nx * p->ny * p->nz;
    for (size_t q = 0; q < n; q++)
        if (p->mat[q] >= p->nmat) return -4;
    return 0;
}

/*
 * Run nsteps reference steps starting at global step t0.  After global step
 * tt, when (tt + 1) % record_every == 0, uz[:, :, 0] (nx*ny values) is stored
 * into surf[((tt + 1) / record_every - 1 - first_record) * nx * ny], where
 * first_record = t0 / record_every.  record_every <= 0 disables recording.
 */
int ora_f64_run(const ora_problem *p, ora_f64_state *s, int t0, int nsteps, int record_every, double *surf,
                int nthreads) {
    int rc = check_problem(p);
    if (rc) return rc;
    if (t0 < 0 || t0 + nsteps > p->nsrc) return -5;
    set_threads(nthreads);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    size_t n123 = (size_t)nx * ny * nz;
    ora_f64_stress T;
    T.T1 = (double *)calloc(n123, sizeof(double));
    T.T2 = (double *)calloc(n123, sizeof(double));
    T.T3 = (double *)calloc(n123, sizeof(double));
    T.T4 = (double *)calloc((size_t)nx * (ny - 1) * (nz - 1), sizeof(double));
    T.T5 = (double *)calloc((size_t)(nx - 1) * ny * (nz - 1), sizeof(double));
    T.T6 = (double *)calloc((size_t)(nx - 1) * (ny - 1) * nz, sizeof(double));
    if (!T.T1 || !T.T2 || !T.T3 || !T.T4 || !T.T5 || !T.T6) {
        free(T.T1); free(T.T2); free(T.T3); free(T.T4); free(T.T5); free(T.T6);
        return -6;
    }
    size_t nux = (size_t)(nx - 1) * ny * nz, nuy = (size_t)nx * (ny - 1) * nz, nuz = (size_t)nx * ny * (nz - 1);
    int first_record = record_every > 0 ? t0 / record_every : 0;
    for (int tt = t0; tt < t0 + nsteps; tt++) {
        apply_source_f64(p, s->uz, tt);
        f64_stress(p, s, &T);
        f64_update(p, s, &T);
        f64_faces(p, s);
        /* time_step: u_old <- u, u <- u_new (u_new keeps its values) */
        memcpy(s->ux_old, s->ux, nux * sizeof(double));
        memcpy(s->uy_old, s->uy, nuy * sizeof(double));
        memcpy(s->uz_old, s->uz, nuz * sizeof(double));
        memcpy(s->ux, s->ux_new, nux * sizeof(double));
        memcpy(s->uy, s->uy_new, nuy * sizeof(double));
        memcpy(s->uz, s->uz_new, nuz * sizeof(double));
        if (record_every > 0 && surf && (tt + 1) % record_every == 0) {
            double *dst = surf + (size_t)((tt + 1) / record_every - 1 - first_record) * nx * ny;
            for (int i = 0; i < nx; i++)
                for (int j = 0; j < ny; j++) dst[(size_t)i * ny + j] = s->uz[I3(ny, nz - 1, i, j, 0)];
        }
    }
    free(T.T1); free(T.T2); free(T.T3); free(T.T4); free(T.T5); free(T.T6);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* (2) FP32 velocity form with Kahan-compensated displacement                */
/* ------------------------------------------------------------------------ */
/*
 * Per-material float constants: C (12) rounded from double, and
 * dtr = (float)(dt / P).  Spacings enter as float reciprocals
 * (float)(1.0 / d).  With e* strains and d* differences:
 *   T1 = fmaf(C00, e1, fmaf(C01, e2, C02 * e3))       (T2, T3 alike)
 *   T4 = C33 * fmaf(duy_dz, ifdz, duz_dy * ifdy)        (T5, T6 alike)
 *   div_x = fmaf(dT1, ifdx, fmaf(dT6, isdy, dT5 * isdz))  (div_y, div_z alike)
 *   v' = fmaf(dtr, div, v);  y = fmaf(dt, v', -c);  t = u + y;
 *   c' = (t - u) - y;  u' = t
 * Faces: u'[b] = fmaf(coef, V - u[b], u[b -/+ 1]) with V the value of the
 * inner neighbour after the earlier faces; v' = c' = 0 there.  Points that the
 * reference never writes keep u, v and c.
 */

typedef struct {
    float *ux, *uy, *uz;
    float *vx, *vy, *vz;
    float *cx, *cy, *cz;
} ora_f32k_state;

typedef struct {
    float c[12];
    float dtr;
} f32mat;

typedef struct {
    float *fdx, *fdy, *fdz, *sdx, *sdy, *sdz; /* reciprocals */
    float fdx0, fdy0, fdz0, sdx0, sdy0, sdz0;
    f32mat *mt;
    float dt;
    float abc[8];
} f32consts;

static void f32_consts(const ora_problem *p, f32consts *k) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    k->fdx = (float *)malloc(sizeof(float) * (nx - 1));
    k->fdy = (float *)malloc(sizeof(float) * (ny - 1));
    k->fdz = (float *)malloc(sizeof(float) * (nz - 1));
    k->sdx = (float *)malloc(sizeof(float) * (nx - 2));
    k->sdy = (float *)malloc(sizeof(float) * (ny - 2));
    k->sdz = (float *)malloc(sizeof(float) * (nz - 2));
    for (int i = 0; i < nx - 1; i++) k->fdx[i] = (float)(1.0 / p->fdx[i]);
    for (int i = 0; i < ny - 1; i++) k->fdy[i] = (float)(1.0 / p->fdy[i]);
    for (int i = 0; i < nz - 1; i++) k->fdz[i] = (float)(1.0 / p->fdz[i]);
    for (int i = 0; i < nx - 2; i++) k->sdx[i] = (float)(1.0 / p->sdx[i]);
    for (int i = 0; i < ny - 2; i++) k->sdy[i] = (float)(1.0 / p->sdy[i]);
    for (int i = 0; i < nz - 2; i++) k->sdz[i] = (float)(1.0 / p->sdz[i]);
    k->fdx0 = k->fdx[0]; k->fdy0 = k->fdy[0]; k->fdz0 = k->fdz[0];
    k->sdx0 = k->sdx[0]; k->sdy0 = k->sdy[0]; k->sdz0 = k->sdz[0];
    k->mt = (f32mat *)malloc(sizeof(f32mat) * p->nmat);
    for (int m = 0; m < p->nmat; m++) {
        const double *t = p->table + (size_t)m * ORA_NTAB;
        for (int q = 0; q < 12; q++) k->mt[m].c[q] = (float)t[q];
        k->mt[m].dtr = (float)(p->dt / t[12]);
    }
    k->dt = (float)p->dt;
    double c[8];
    ora_abc_coeffs(p, c);
    for (int q = 0; q < 8; q++) k->abc[q] = p->bc == 1 ? 0.0f : (float)c[q];
}

static void f32_consts_free(f32consts *k) {
    free(k->fdx); free(k->fdy); free(k->fdz); free(k->sdx); free(k->sdy); free(k->sdz); free(k->mt);
}

typedef struct {
    float *T1, *T2, *T3, *T4, *T5, *T6;
} f32stress;

/* u read with the source substituted on the x=0 plane of uz */
static inline float uzs(const ora_problem *p, const float *uz, float s, int i, int j, int k) {
    if (i == 0 && (p->source_mode == 1 || k == 0)) return s;
    return uz[I3(p->ny, p->nz - 1, i, j, k)];
}

static void f32_stress(const ora_problem *p, const f32consts *K, const ora_f32k_state *s, float src, f32stress *T) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const float *ux = s->ux, *uy = s->uy, *uz = s->uz;
    const uint8_t *mat = p->mat;
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                const float *c = K->mt[mat[I3(ny, nz, i, j, k)]].c;
                float dux = ux[I3(ny, nz, i, j, k)] - ux[I3(ny, nz, i - 1, j, k)];
                float duy = uy[I3(ny - 1, nz, i, j, k)] - uy[I3(ny - 1, nz, i, j - 1, k)];
                float e1, e2, e3;
                if (k == 0) {
                    float duz = uzs(p, uz, src, i, j, 0);
                    e1 = dux * K->sdx0; e2 = duy * K->sdy0; e3 = duz * K->sdz0;
                } else {
                    float duz = uzs(p, uz, src, i, j, k) - uzs(p, uz, src, i, j, k - 1);
                    e1 = dux * K->sdx[i - 1]; e2 = duy * K->sdy[j - 1]; e3 = duz * K->sdz[k - 1];
                }
                size_t o = I3(ny, nz, i, j, k);
                T->T1[o] = fmaf(c[0], e1, fmaf(c[1], e2, c[2] * e3));
                T->T2[o] = fmaf(c[3], e1, fmaf(c[4], e2, c[5] * e3));
                T->T3[o] = k == 0 ? 0.0f : fmaf(c[6], e1, fmaf(c[7], e2, c[8] * e3));
            }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                float a = uy[I3(ny - 1, nz, i, j, k + 1)] - uy[I3(ny - 1, nz, i, j, k)];
                float b = uzs(p, uz, src, i, j + 1, k) - uzs(p, uz, src, i, j, k);
                float v;
                if (k == 0) v = K->mt[mat[I3(ny, nz, i, j + 1, 0)]].c[9] * fmaf(a, K->fdy0, b * K->fdz0);
                else v = K->mt[mat[I3(ny, nz, i, j + 1, k + 1)]].c[9] * fmaf(a, K->fdz[k], b * K->fdy[j]);
                T->T4[I3(ny - 1, nz - 1, i, j, k)] = v;
            }
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                float a = ux[I3(ny, nz, i, j, k + 1)] - ux[I3(ny, nz, i, j, k)];
                float b = uzs(p, uz, src, i + 1, j, k) - uzs(p, uz, src, i, j, k);
                float v;
                if (k == 0) v = K->mt[mat[I3(ny, nz, i + 1, j, 0)]].c[10] * fmaf(a, K->fdx0, b * K->fdz0);
                else v = K->mt[mat[I3(ny, nz, i + 1, j, k + 1)]].c[10] * fmaf(a, K->fdz[k], b * K->fdx[i]);
                T->T5[I3(ny, nz - 1, i, j, k)] = v;
            }
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                float a = ux[I3(ny, nz, i, j + 1, k)] - ux[I3(ny, nz, i, j, k)];
                float b = uy[I3(ny - 1, nz, i + 1, j, k)] - uy[I3(ny - 1, nz, i, j, k)];
                float v;
                if (k == 0) v = K->mt[mat[I3(ny, nz, i + 1, j + 1, 0)]].c[11] * fmaf(a, K->fdx0, b * K->fdz0);
                else v = K->mt[mat[I3(ny, nz, i + 1, j + 1, k)]].c[11] * fmaf(a, K->fdy[j], b * K->fdx[i]);
                T->T6[I3(ny - 1, nz, i, j, k)] = v;
            }
}

static inline void kahan(float u, float v, float c, float dtr, float div, float dt, float *u2, float *v2, float *c2) {
    float vn = fmaf(dtr, div, v);
    float y = fmaf(dt, vn, -c);
    float t = u + y;
    *c2 = (t - u) - y;
    *v2 = vn;
    *u2 = t;
}

static void f32_update(const ora_problem *p, const f32consts *K, const ora_f32k_state *s, ora_f32k_state *o,
                       const f32stress *T) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const uint8_t *mat = p->mat;
    const float dt = K->dt;
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                float d1 = T->T1[I3(ny, nz, i + 1, j, k)] - T->T1[I3(ny, nz, i, j, k)];
                float d6 = T->T6[I3(ny - 1, nz, i, j, k)] - T->T6[I3(ny - 1, nz, i, j - 1, k)];
                float div, dtr;
                if (k == 0) {
                    float d5 = T->T5[I3(ny, nz - 1, i, j, 0)];
                    div = fmaf(d1, K->fdx0, fmaf(d6, K->sdy0, d5 * K->sdz0));
                    dtr = K->mt[mat[I3(ny, nz, i + 1, j, 0)]].dtr;
                } else {
                    float d5 = T->T5[I3(ny, nz - 1, i, j, k)] - T->T5[I3(ny, nz - 1, i, j, k - 1)];
                    div = fmaf(d1, K->fdx[i], fmaf(d6, K->sdy[j - 1], d5 * K->sdz[k - 1]));
                    dtr = K->mt[mat[I3(ny, nz, i + 1, j, k)]].dtr;
                }
                size_t q = I3(ny, nz, i, j, k);
                kahan(s->ux[q], s->vx[q], s->cx[q], dtr, div, dt, &o->ux[q], &o->vx[q], &o->cx[q]);
            }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 0; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                float d6 = T->T6[I3(ny - 1, nz, i, j, k)] - T->T6[I3(ny - 1, nz, i - 1, j, k)];
                float d2 = T->T2[I3(ny, nz, i, j + 1, k)] - T->T2[I3(ny, nz, i, j, k)];
                float div, dtr;
                if (k == 0) {
                    float d4 = T->T4[I3(ny - 1, nz - 1, i, j, 0)];
                    div = fmaf(d6, K->sdx0, fmaf(d2, K->fdy0, d4 * K->sdz0));
                    dtr = K->mt[mat[I3(ny, nz, i, j + 1, 0)]].dtr;
                } else {
                    float d4 = T->T4[I3(ny - 1, nz - 1, i, j, k)] - T->T4[I3(ny - 1, nz - 1, i, j, k - 1)];
                    div = fmaf(d6, K->sdx[i - 1], fmaf(d2, K->fdy[j], d4 * K->sdz[k - 1]));
                    dtr = K->mt[mat[I3(ny, nz, i, j + 1, k)]].dtr;
                }
                size_t q = I3(ny - 1, nz, i, j, k);
                kahan(s->uy[q], s->vy[q], s->cy[q], dtr, div, dt, &o->uy[q], &o->vy[q], &o->cy[q]);
            }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx - 2; i++)
        for (int j = 1; j <= ny - 2; j++)
            for (int k = 0; k <= nz - 2; k++) {
                float d5 = T->T5[I3(ny, nz - 1, i, j, k)] - T->T5[I3(ny, nz - 1, i - 1, j, k)];
                float d4 = T->T4[I3(ny - 1, nz - 1, i, j, k)] - T->T4[I3(ny - 1, nz - 1, i, j - 1, k)];
                float t3n = T->T3[I3(ny, nz, i, j, k + 1)];
                float div, dtr;
                if (k == 0) {
                    if (p->surface_mode == 0) div = fmaf(d5, K->sdx0, d4 * K->sdy0) + t3n;
                    else div = fmaf(d5, K->sdx0, fmaf(d4, K->sdy0, t3n * K->fdz0));
                    dtr = K->mt[mat[I3(ny, nz, i, j, 0)]].dtr;
                } else {
                    float d3 = t3n - T->T3[I3(ny, nz, i, j, k)];
                    div = fmaf(d5, K->sdx[i - 1], fmaf(d4, K->sdy[j - 1], d3 * K->fdz[k]));
                    dtr = K->mt[mat[I3(ny, nz, i, j, k + 1)]].dtr;
                }
                size_t q = I3(ny, nz - 1, i, j, k);
                kahan(s->uz[q], s->vz[q], s->cz[q], dtr, div, dt, &o->uz[q], &o->vz[q], &o->cz[q]);
            }
}

/* f32 faces: o holds the new state with every non-face point already final. */
static void f32_faces(const ora_problem *p, const f32consts *K, const ora_f32k_state *s, ora_f32k_state *o,
                      float src) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const float *ux = s->ux, *uy = s->uy, *uz = s->uz;
    float *xn = o->ux, *yn = o->uy, *zn = o->uz;
    const float *c = K->abc;
    const int rigid = p->bc == 1;
#define F32ABC(dst, nbr_new, nbr_old, self_old, coef) \
    (dst) = rigid ? 0.0f : fmaf((coef), (nbr_new) - (self_old), (nbr_old))
    for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz; k++)
            F32ABC(xn[I3(ny, nz, nx - 2, j, k)], xn[I3(ny, nz, nx - 3, j, k)], ux[I3(ny, nz, nx - 3, j, k)],
                   ux[I3(ny, nz, nx - 2, j, k)], c[0]);
    for (int j = 0; j < ny - 1; j++)
        for (int k = 0; k < nz; k++)
            F32ABC(yn[I3(ny - 1, nz, nx - 1, j, k)], yn[I3(ny - 1, nz, nx - 2, j, k)],
                   uy[I3(ny - 1, nz, nx - 2, j, k)], uy[I3(ny - 1, nz, nx - 1, j, k)], c[1]);
    for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz - 1; k++)
            F32ABC(zn[I3(ny, nz - 1, nx - 1, j, k)], zn[I3(ny, nz - 1, nx - 2, j, k)],
                   uzs(p, uz, src, nx - 2, j, k), uzs(p, uz, src, nx - 1, j, k), c[1]);
    for (int i = 0; i < nx - 1; i++)
        for (int k = 0; k < nz; k++)
            F32ABC(xn[I3(ny, nz, i, 0, k)], xn[I3(ny, nz, i, 1, k)], ux[I3(ny, nz, i, 1, k)], ux[I3(ny, nz, i, 0, k)],
                   c[2]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz; k++)
            F32ABC(yn[I3(ny - 1, nz, i, 0, k)], yn[I3(ny - 1, nz, i, 1, k)], uy[I3(ny - 1, nz, i, 1, k)],
                   uy[I3(ny - 1, nz, i, 0, k)], c[3]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz - 1; k++)
            F32ABC(zn[I3(ny, nz - 1, i, 0, k)], zn[I3(ny, nz - 1, i, 1, k)], uzs(p, uz, src, i, 1, k),
                   uzs(p, uz, src, i, 0, k), c[2]);
    for (int i = 0; i < nx - 1; i++)
        for (int k = 0; k < nz; k++)
            F32ABC(xn[I3(ny, nz, i, ny - 1, k)], xn[I3(ny, nz, i, ny - 2, k)], ux[I3(ny, nz, i, ny - 2, k)],
                   ux[I3(ny, nz, i, ny - 1, k)], c[4]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz; k++)
            F32ABC(yn[I3(ny - 1, nz, i, ny - 2, k)], yn[I3(ny - 1, nz, i, ny - 3, k)],
                   uy[I3(ny - 1, nz, i, ny - 3, k)], uy[I3(ny - 1, nz, i, ny - 2, k)], c[5]);
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz - 1; k++)
            F32ABC(zn[I3(ny, nz - 1, i, ny - 1, k)], zn[I3(ny, nz - 1, i, ny - 2, k)],
                   uzs(p, uz, src, i, ny - 2, k), uzs(p, uz, src, i, ny - 1, k), c[4]);
    for (int i = 0; i < nx - 1; i++)
        for (int j = 0; j < ny; j++)
            F32ABC(xn[I3(ny, nz, i, j, nz - 1)], xn[I3(ny, nz, i, j, nz - 2)], ux[I3(ny, nz, i, j, nz - 2)],
                   ux[I3(ny, nz, i, j, nz - 1)], c[6]);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny - 1; j++)
            F32ABC(yn[I3(ny - 1, nz, i, j, nz - 1)], yn[I3(ny - 1, nz, i, j, nz - 2)],
                   uy[I3(ny - 1, nz, i, j, nz - 2)], uy[I3(ny - 1, nz, i, j, nz - 1)], c[6]);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            F32ABC(zn[I3(ny, nz - 1, i, j, nz - 2)], zn[I3(ny, nz - 1, i, j, nz - 3)],
                   uzs(p, uz, src, i, j, nz - 3), uzs(p, uz, src, i, j, nz - 2), c[7]);
#undef F32ABC
}

/* face predicates of the reference's four absorbing faces */
static inline int on_face_x(const ora_problem *p, int comp, int i) { return i == (comp == 0 ? p->nx - 2 : p->nx - 1); }
static inline int on_face_y(const ora_problem *p, int comp, int j) {
    return j == 0 || j == (comp == 1 ? p->ny - 2 : p->ny - 1);
}
static inline int on_face_z(const ora_problem *p, int comp, int k) { return k == (comp == 2 ? p->nz - 2 : p->nz - 1); }

static void f32_zero_faces_vc(const ora_problem *p, ora_f32k_state *o) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    for (int comp = 0; comp < 3; comp++) {
        int ex = nx - (comp == 0), ey = ny - (comp == 1), ez = nz - (comp == 2);
        float *v = comp == 0 ? o->vx : comp == 1 ? o->vy : o->vz;
        float *c = comp == 0 ? o->cx : comp == 1 ? o->cy : o->cz;
        for (int i = 0; i < ex; i++)
            for (int j = 0; j < ey; j++)
                for (int k = 0; k < ez; k++)
                    if (on_face_x(p, comp, i) || on_face_y(p, comp, j) || on_face_z(p, comp, k)) {
                        v[I3(ey, ez, i, j, k)] = 0.0f;
                        c[I3(ey, ez, i, j, k)] = 0.0f;
                    }
    }
}

int ora_f32k_run(const ora_problem *p, ora_f32k_state *s, int t0, int nsteps, int record_every, float *surf,
                 int nthreads) {
    int rc = check_problem(p);
    if (rc) return rc;
    if (t0 < 0 || t0 + nsteps > p->nsrc) return -5;
    set_threads(nthreads);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    size_t n123 = (size_t)nx * ny * nz;
    size_t nux = (size_t)(nx - 1) * ny * nz, nuy = (size_t)nx * (ny - 1) * nz, nuz = (size_t)nx * ny * (nz - 1);
    f32consts K;
    f32_consts(p, &K);
    f32stress T;
    T.T1 = (float *)calloc(n123, sizeof(float));
    T.T2 = (float *)calloc(n123, sizeof(float));
    T.T3 = (float *)calloc(n123, sizeof(float));
    T.T4 = (float *)calloc((size_t)nx * (ny - 1) * (nz - 1), sizeof(float));
    T.T5 = (float *)calloc((size_t)(nx - 1) * ny * (nz - 1), sizeof(float));
    T.T6 = (float *)calloc((size_t)(nx - 1) * (ny - 1) * nz, sizeof(float));
    ora_f32k_state o;
    size_t sz[3] = {nux, nuy, nuz};
    float **dst[9] = {&o.ux, &o.uy, &o.uz, &o.vx, &o.vy, &o.vz, &o.cx, &o.cy, &o.cz};
    float *srcp[9] = {s->ux, s->uy, s->uz, s->vx, s->vy, s->vz, s->cx, s->cy, s->cz};
    for (int q = 0; q < 9; q++) *dst[q] = (float *)malloc(sz[q % 3] * sizeof(float));
    int first_record = record_every > 0 ? t0 / record_every : 0;
    for (int tt = t0; tt < t0 + nsteps; tt++) {
        float src = (float)p->src[tt];
        /* stale copy: points the reference never writes keep their state */
        for (int q = 0; q < 9; q++) memcpy(*dst[q], srcp[q], sz[q % 3] * sizeof(float));
        f32_stress(p, &K, s, src, &T);
        f32_update(p, &K, s, &o, &T);
        f32_faces(p, &K, s, &o, src);
        f32_zero_faces_vc(p, &o);
        for (int q = 0; q < 9; q++) memcpy(srcp[q], *dst[q], sz[q % 3] * sizeof(float));
        if (record_every > 0 && surf && (tt + 1) % record_every == 0) {
            float *d = surf + (size_t)((tt + 1) / record_every - 1 - first_record) * nx * ny;
            for (int i = 0; i < nx; i++)
                for (int j = 0; j < ny; j++) d[(size_t)i * ny + j] = s->uz[I3(ny, nz - 1, i, j, 0)];
        }
    }
    for (int q = 0; q < 9; q++) free(*dst[q]);
    free(T.T1); free(T.T2); free(T.T3); free(T.T4); free(T.T5); free(T.T6);
    f32_consts_free(&K);
    return 0;
}
