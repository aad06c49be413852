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

/* face predicates of the reference's four absorbing faces */
static inline int on_face_x(const ora_problem *p, int comp, int i) { return i == (comp == 0 ? p->nx - 2 : p->nx - 1); }
static inline int on_face_y(const ora_problem *p, int comp, int j) {
    return j == 0 || j == (comp == 1 ? p->ny - 2 : p->ny - 1);
}
static inline int on_face_z(const ora_problem *p, int comp, int k) { return k == (comp == 2 ? p->nz - 2 : p->nz - 1); }


/* ------------------------------------------------------------------------ */
/* (2) velocity form with Kahan-compensated displacement: FP32 and FP64      */
/* ------------------------------------------------------------------------ */
#define REAL float
#define FMA fmaf
#define V(name) name##_f32k
#include "velocity_form.inc"
#undef REAL
#undef FMA
#undef V

#define REAL double
#define FMA fma
#define V(name) name##_f64v
#include "velocity_form.inc"
#undef REAL
#undef FMA
#undef V
