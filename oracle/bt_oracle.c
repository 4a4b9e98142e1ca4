/*
 * Oracle for the Bloch–Torrey step — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP64 restatement of the reference solver's CPU path, used as the
 * checker by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py. The product (initializator_gb300/) never links or calls it.
 *
 * Followed reference functions (paths relative to the reference project):
 *   ExplicitSimple                src/NmrRelaxationSolve.cpp:3148-3282  (the update)
 *   FillInDiffusinAndTime         src/NmrRelaxationSolve.cpp:1756-1841  (D, T1, T2 per voxel)
 *   BoundaryConditionsForActiveCells / ForDiffusion / ForVectorField
 *                                 src/NmrRelaxationSolve.cpp:880-928, 1895-1942, 1664-1754
 *                                 (one rank: every ghost layer is a copy of its neighbour)
 *   FillInMainField               src/NmrRelaxationSolve.cpp:1944-1972  (noise = G*d*(i-0.5))
 *   OrtTransform / AddImpulse     src/NmrRelaxationSolve.cpp:2536-2608
 *   OutputX/Y/Z (NCOMP = 1)       src/NmrRelaxationSolve.cpp:3301-3461
 *
 * The arrays carry one ghost layer exactly like the reference
 * (idx = i + (nx+2)*(j + (ny+2)*k), cpp:3284-3287), and every expression keeps
 * the reference's operation order, so with -ffp-contract=off the field is
 * bit-identical to the reference's for the same inputs. The only deliberate
 * difference: M(t) sums are taken per z-plane and then added plane by plane
 * (deterministic for any thread count) instead of one running sum.
 *
 * Parity of this restatement is pinned against the reference itself
 * (oracle/_ref, built from the reference sources by oracle/Makefile) through
 * the fixtures in tests/golden/.
 */
#include "bt_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double g_loop_seconds = 0.0;

/* wall time of the stepping loop of the last bto_run_reference call (set-up of
 * the ghosted arrays excluded), for timing the CPU baseline */
double bto_last_loop_seconds(void) { return g_loop_seconds; }

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#define SMALL 1.0e-50
#define BIG 1.0e+50

typedef struct {
    int nx, ny, nz;
    size_t sx, sy, num;  /* strides of the ghosted layout */
} grid_t;

static inline size_t gidx(const grid_t* g, int i, int j, int k) {
    return (size_t)i + g->sx * (size_t)j + g->sy * (size_t)k;
}

/* ghost layers by copying the neighbouring interior/edge value, x then y then z,
 * each over the full extent of the other two axes (cpp:1666-1753 at one rank) */
static void bc_copy_d(const grid_t* g, double* f) {
    int nx = g->nx, ny = g->ny, nz = g->nz;
    for (int k = 0; k < nz + 2; k++)
        for (int j = 0; j < ny + 2; j++) {
            f[gidx(g, 0, j, k)] = f[gidx(g, 1, j, k)];
            f[gidx(g, nx + 1, j, k)] = f[gidx(g, nx, j, k)];
        }
    for (int k = 0; k < nz + 2; k++)
        for (int i = 0; i < nx + 2; i++) {
            f[gidx(g, i, 0, k)] = f[gidx(g, i, 1, k)];
            f[gidx(g, i, ny + 1, k)] = f[gidx(g, i, ny, k)];
        }
    for (int j = 0; j < ny + 2; j++)
        for (int i = 0; i < nx + 2; i++) {
            f[gidx(g, i, j, 0)] = f[gidx(g, i, j, 1)];
            f[gidx(g, i, j, nz + 1)] = f[gidx(g, i, j, nz)];
        }
}

/* ghost layers per axis (x, then y, then z, each over the full extent of the
 * other two axes): 0 copy of the neighbouring cell (BC_ZeroDer_*,
 * src/NmrRelaxationSolveKernels.cu:969-1000), 1 periodic, the far interior
 * plane (BC_Inf_*, cu:1002-1033), 2 zero (BC_Advanced_XM/XP with Val 0,
 * cu:1035-1053; the GPU path also leaves zero in the ghosts of a pair it does
 * not handle, cu:1321-1396) */
static void bc_apply_d(const grid_t* g, double* f, const int mode[3]) {
    int nx = g->nx, ny = g->ny, nz = g->nz;
    for (int k = 0; k < nz + 2; k++)
        for (int j = 0; j < ny + 2; j++) {
            size_t lo = gidx(g, 0, j, k), hi = gidx(g, nx + 1, j, k);
            if (mode[0] == 1) { f[lo] = f[gidx(g, nx, j, k)]; f[hi] = f[gidx(g, 1, j, k)]; }
            else if (mode[0] == 2) { f[lo] = 0.0; f[hi] = 0.0; }
            else { f[lo] = f[gidx(g, 1, j, k)]; f[hi] = f[gidx(g, nx, j, k)]; }
        }
    for (int k = 0; k < nz + 2; k++)
        for (int i = 0; i < nx + 2; i++) {
            size_t lo = gidx(g, i, 0, k), hi = gidx(g, i, ny + 1, k);
            if (mode[1] == 1) { f[lo] = f[gidx(g, i, ny, k)]; f[hi] = f[gidx(g, i, 1, k)]; }
            else if (mode[1] == 2) { f[lo] = 0.0; f[hi] = 0.0; }
            else { f[lo] = f[gidx(g, i, 1, k)]; f[hi] = f[gidx(g, i, ny, k)]; }
        }
    for (int j = 0; j < ny + 2; j++)
        for (int i = 0; i < nx + 2; i++) {
            size_t lo = gidx(g, i, j, 0), hi = gidx(g, i, j, nz + 1);
            if (mode[2] == 1) { f[lo] = f[gidx(g, i, j, nz)]; f[hi] = f[gidx(g, i, j, 1)]; }
            else if (mode[2] == 2) { f[lo] = 0.0; f[hi] = 0.0; }
            else { f[lo] = f[gidx(g, i, j, 1)]; f[hi] = f[gidx(g, i, j, nz)]; }
        }
}

static void bc_copy_c(const grid_t* g, char* f) {
    int nx = g->nx, ny = g->ny, nz = g->nz;
    for (int k = 0; k < nz + 2; k++)
        for (int j = 0; j < ny + 2; j++) {
            f[gidx(g, 0, j, k)] = f[gidx(g, 1, j, k)];
            f[gidx(g, nx + 1, j, k)] = f[gidx(g, nx, j, k)];
        }
    for (int k = 0; k < nz + 2; k++)
        for (int i = 0; i < nx + 2; i++) {
            f[gidx(g, i, 0, k)] = f[gidx(g, i, 1, k)];
            f[gidx(g, i, ny + 1, k)] = f[gidx(g, i, ny, k)];
        }
    for (int j = 0; j < ny + 2; j++)
        for (int i = 0; i < nx + 2; i++) {
            f[gidx(g, i, j, 0)] = f[gidx(g, i, j, 1)];
            f[gidx(g, i, j, nz + 1)] = f[gidx(g, i, j, nz)];
        }
}

typedef struct {
    grid_t g;
    char* act;
    double *D, *t1, *t2;
    double *vx, *vy, *vz;
    double *mx, *my, *mz, *ax, *ay, *az;
} ofields_t;

static void ofields_free(ofields_t* f) {
    free(f->act); free(f->D); free(f->t1); free(f->t2);
    free(f->vx); free(f->vy); free(f->vz);
    free(f->mx); free(f->my); free(f->mz);
    free(f->ax); free(f->ay); free(f->az);
}

/* FillInDiffusinAndTime for one component of fluid (c1 = 1, c2 = 0): the
 * bulk rate plus rho/d for every solid face neighbour, in the order
 * -x, +x, -y, +y, -z, +z; T = 1/rate; solid voxels get D = 1e-50, T = 1e50. */
static void fill_coeffs(const bto_params* p, ofields_t* f) {
    const grid_t* g = &f->g;
    for (int k = 1; k <= g->nz; k++)
        for (int j = 1; j <= g->ny; j++)
            for (int i = 1; i <= g->nx; i++) {
                size_t c = gidx(g, i, j, k);
                if (f->act[c] == 0) {
                    f->D[c] = SMALL;
                    f->t1[c] = BIG;
                    f->t2[c] = BIG;
                    continue;
                }
                double ct1 = 1.0 / p->t1;
                double ct2 = 1.0 / p->t2;
                if (f->act[gidx(g, i - 1, j, k)] == 0) { ct1 += p->rho1 / p->dx; ct2 += p->rho2 / p->dx; }
                if (f->act[gidx(g, i + 1, j, k)] == 0) { ct1 += p->rho1 / p->dx; ct2 += p->rho2 / p->dx; }
                if (f->act[gidx(g, i, j - 1, k)] == 0) { ct1 += p->rho1 / p->dy; ct2 += p->rho2 / p->dy; }
                if (f->act[gidx(g, i, j + 1, k)] == 0) { ct1 += p->rho1 / p->dy; ct2 += p->rho2 / p->dy; }
                if (f->act[gidx(g, i, j, k - 1)] == 0) { ct1 += p->rho1 / p->dz; ct2 += p->rho2 / p->dz; }
                if (f->act[gidx(g, i, j, k + 1)] == 0) { ct1 += p->rho1 / p->dz; ct2 += p->rho2 / p->dz; }
                f->D[c] = p->diffusion ? p->d_pore : SMALL;
                f->t1[c] = 1.0 / ct1;
                f->t2[c] = 1.0 / ct2;
            }
    bc_copy_d(g, f->D);
}

static int ofields_init(const bto_params* p, const uint8_t* mask,
                        const double* vx, const double* vy, const double* vz,
                        const double* mx, const double* my, const double* mz,
                        ofields_t* f) {
    memset(f, 0, sizeof(*f));
    grid_t* g = &f->g;
    g->nx = p->nx; g->ny = p->ny; g->nz = p->nz;
    g->sx = (size_t)(p->nx + 2);
    g->sy = g->sx * (size_t)(p->ny + 2);
    g->num = g->sy * (size_t)(p->nz + 2);
    f->act = (char*)calloc(g->num, 1);
    double** arrs[] = {&f->D, &f->t1, &f->t2, &f->vx, &f->vy, &f->vz,
                       &f->mx, &f->my, &f->mz, &f->ax, &f->ay, &f->az};
    for (size_t a = 0; a < sizeof(arrs) / sizeof(arrs[0]); a++)
        *arrs[a] = (double*)calloc(g->num, sizeof(double));
    if (!f->act || !f->az) { ofields_free(f); return -1; }
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t s = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                size_t c = gidx(g, i + 1, j + 1, k + 1);
                f->act[c] = mask[s] ? 1 : 0;
                f->mx[c] = mx[s]; f->my[c] = my[s]; f->mz[c] = mz[s];
            }
    bc_copy_c(g, f->act);
    fill_coeffs(p, f);
    /* ReadVelocity (cpp:1435-1536): face i of cell i sits at ghosted index i+1 */
    if (vx && vy && vz) {
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i <= nx; i++)
                    f->vx[gidx(g, i + 1, j + 1, k + 1)] = vx[(size_t)i + (size_t)(nx + 1) * ((size_t)j + (size_t)ny * k)];
        for (int k = 0; k < nz; k++)
            for (int j = 0; j <= ny; j++)
                for (int i = 0; i < nx; i++)
                    f->vy[gidx(g, i + 1, j + 1, k + 1)] = vy[(size_t)i + (size_t)nx * ((size_t)j + (size_t)(ny + 1) * k)];
        for (int k = 0; k <= nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++)
                    f->vz[gidx(g, i + 1, j + 1, k + 1)] = vz[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)];
    }
    bc_copy_d(g, f->mx); bc_copy_d(g, f->my); bc_copy_d(g, f->mz);
    return 0;
}

/* ExplicitSimple (cpp:3148-3282) for the z-plane k of the ghosted arrays. */
static void update_plane(const bto_params* p, const ofields_t* f, int k, const double G[3]) {
    const grid_t* g = &f->g;
    const double dTime = p->dt;
    const double hx = dTime / p->dx, hy = dTime / p->dy, hz = dTime / p->dz;
    const double hxx = dTime / (p->dx * p->dx), hyy = dTime / (p->dy * p->dy), hzz = dTime / (p->dz * p->dz);
    const double* D = f->D;
    const double *mX = f->mx, *mY = f->my, *mZ = f->mz;
    const double Bx = p->main_field[0], By = p->main_field[1], Bz = p->main_field[2];
    const int km = k - 1, kp = k + 1;
    for (int j = 1; j <= g->ny; j++) {
        const int jm = j - 1, jp = j + 1;
        for (int i = 1; i <= g->nx; i++) {
            const int im = i - 1, ip = i + 1;
            const size_t c = gidx(g, i, j, k);
            if (f->act[c] != 1) continue;
            const size_t cxp = gidx(g, ip, j, k), cxm = gidx(g, im, j, k);
            const size_t cyp = gidx(g, i, jp, k), cym = gidx(g, i, jm, k);
            const size_t czp = gidx(g, i, j, kp), czm = gidx(g, i, j, km);
            double tau1 = 1.0 / f->t1[c];
            double tau2 = 1.0 / f->t2[c];
            double dxp = 2.0 * (D[cxp] * D[c]) / (D[cxp] + D[c] + SMALL);
            double dxm = 2.0 * (D[cxm] * D[c]) / (D[cxm] + D[c] + SMALL);
            double dyp = 2.0 * (D[cyp] * D[c]) / (D[cyp] + D[c] + SMALL);
            double dym = 2.0 * (D[cym] * D[c]) / (D[cym] + D[c] + SMALL);
            double dzp = 2.0 * (D[czp] * D[c]) / (D[czp] + D[c] + SMALL);
            double dzm = 2.0 * (D[czm] * D[c]) / (D[czm] + D[c] + SMALL);
            double px0 = mX[c], py0 = mY[c], pz0 = mZ[c];
            double um = f->vx[c], umm = um / (um + SMALL);
            double vm = f->vy[c], vmm = vm / (vm + SMALL);
            double wm = f->vz[c], wmm = wm / (wm + SMALL);
            double up = f->vx[cxp], upp = up / (up + SMALL);
            double vp = f->vy[cyp], vpp = vp / (vp + SMALL);
            double wp = f->vz[czp], wpp = wp / (wp + SMALL);
            double u = 0.5 * (um + up), v = 0.5 * (vm + vp), w = 0.5 * (wm + wp);
            double ud = fabs(u), vd = fabs(v), wd = fabs(w);
            double anb = sqrt(Bx * Bx + By * By + Bz * Bz);
            double anx = Bx / anb, any = By / anb, anz = Bz / anb;
            double pEq = p->p_eq;
            double pxEq = pEq * anx, pyEq = pEq * any, pzEq = pEq * anz;
            double div = anx * px0 + any * py0 + anz * pz0;
            double divx = anx * div, divy = any * div, divz = anz * div;
            double b = dTime * p->gamma;
            /* FillInMainField noise field: G * d * (i - 0.5), ghosted 1-based index */
            double bbxb = b * (G[0] * p->dx * ((double)i - 0.5));
            double bbyb = b * (G[1] * p->dy * ((double)j - 0.5));
            double bbzb = b * (G[2] * p->dz * ((double)k - 0.5));
            double ax = px0 + dTime * tau1 * (pxEq - divx) + dTime * tau2 * (divx - px0);
            double ay = py0 + dTime * tau1 * (pyEq - divy) + dTime * tau2 * (divy - py0);
            double az = pz0 + dTime * tau1 * (pzEq - divz) + dTime * tau2 * (divz - pz0);
            if (p->vector_mult == 1) {
                ax += 0.0 - bbyb * pz0 + bbzb * py0;
                ay += 0.0 + bbxb * pz0 - bbzb * px0;
                az += 0.0 - bbxb * py0 + bbyb * px0;
            }
            if (p->velocity == 1) {
                ax -= 0.5 * hx * ((u - ud) * (mX[cxp] - px0) * upp + (u + ud) * (px0 - mX[cxm]) * umm)
                    + 0.5 * hy * ((v - vd) * (mX[cyp] - px0) * vpp + (v + vd) * (px0 - mX[cym]) * vmm)
                    + 0.5 * hz * ((w - wd) * (mX[czp] - px0) * wpp + (w + wd) * (px0 - mX[czm]) * wmm);
                ay -= 0.5 * hx * ((u - ud) * (mY[cxp] - py0) * upp + (u + ud) * (py0 - mY[cxm]) * umm)
                    + 0.5 * hy * ((v - vd) * (mY[cyp] - py0) * vpp + (v + vd) * (py0 - mY[cym]) * vmm)
                    + 0.5 * hz * ((w - wd) * (mY[czp] - py0) * wpp + (w + wd) * (py0 - mY[czm]) * wmm);
                az -= 0.5 * hx * ((u - ud) * (mZ[cxp] - pz0) * upp + (u + ud) * (pz0 - mZ[cxm]) * umm)
                    + 0.5 * hy * ((v - vd) * (mZ[cyp] - pz0) * vpp + (v + vd) * (pz0 - mZ[cym]) * vmm)
                    + 0.5 * hz * ((w - wd) * (mZ[czp] - pz0) * wpp + (w + wd) * (pz0 - mZ[czm]) * wmm);
            }
            if (p->diffusion == 1) {
                ax += hxx * (dxp * (mX[cxp] - px0) - dxm * (px0 - mX[cxm]))
                    + hyy * (dyp * (mX[cyp] - px0) - dym * (px0 - mX[cym]))
                    + hzz * (dzp * (mX[czp] - px0) - dzm * (px0 - mX[czm]));
                ay += hxx * (dxp * (mY[cxp] - py0) - dxm * (py0 - mY[cxm]))
                    + hyy * (dyp * (mY[cyp] - py0) - dym * (py0 - mY[cym]))
                    + hzz * (dzp * (mY[czp] - py0) - dzm * (py0 - mY[czm]));
                az += hxx * (dxp * (mZ[cxp] - pz0) - dxm * (pz0 - mZ[cxm]))
                    + hyy * (dyp * (mZ[cyp] - pz0) - dym * (pz0 - mZ[cym]))
                    + hzz * (dzp * (mZ[czp] - pz0) - dzm * (pz0 - mZ[czm]));
            }
            f->ax[c] = ax; f->ay[c] = ay; f->az[c] = az;
        }
    }
}

/* One stage of the reference's GPU scheme, MacCormack predictor-corrector
 * (ExplicitMakUpgrade cu:1473-1498): stage 0 = NMR_predictor_upgrade
 * (cu:637-801) from the field M into P, stage 1 = NMR_corrector_upgrade
 * (cu:803-967) from P into the corrected field. Relaxation, cross product and
 * diffusion (face diffusivity 2DaDb/(Da+Db+1e-25)) act on the stage's input;
 * advection uses the cell-average velocity with backward differences in the
 * predictor and forward differences in the corrector. A solid neighbour in an
 * advective difference holds the voxel's own value (the reference writes it
 * there first; with several writers the GPU's pick is racy, this is the
 * zero-flux reading). Corrector: out = 0.5 * (M + P + the terms of P), summed
 * in the reference's order. */
static void mac_plane(const bto_params* p, const ofields_t* f, int k, const double G[3], int stage,
                      const double* iX, const double* iY, const double* iZ, double* oX, double* oY, double* oZ) {
    const grid_t* g = &f->g;
    const double dTime = p->dt;
    const double hx = dTime / p->dx, hy = dTime / p->dy, hz = dTime / p->dz;
    const double hxx = dTime / (p->dx * p->dx), hyy = dTime / (p->dy * p->dy), hzz = dTime / (p->dz * p->dz);
    const double* D = f->D;
    const double Bx = p->main_field[0], By = p->main_field[1], Bz = p->main_field[2];
    const double reg = 1.0e-25;
    const int km = k - 1, kp = k + 1;
    for (int j = 1; j <= g->ny; j++) {
        const int jm = j - 1, jp = j + 1;
        for (int i = 1; i <= g->nx; i++) {
            const int im = i - 1, ip = i + 1;
            const size_t c = gidx(g, i, j, k);
            if (f->act[c] != 1) continue;
            const size_t cxp = gidx(g, ip, j, k), cxm = gidx(g, im, j, k);
            const size_t cyp = gidx(g, i, jp, k), cym = gidx(g, i, jm, k);
            const size_t czp = gidx(g, i, j, kp), czm = gidx(g, i, j, km);
            const double* in[3] = {iX, iY, iZ};
            const double p0[3] = {iX[c], iY[c], iZ[c]};
            const double tau1 = 1.0 / f->t1[c];
            const double tau2 = 1.0 / f->t2[c];
            const double anb = sqrt(Bx * Bx + By * By + Bz * Bz);
            const double an[3] = {Bx / anb, By / anb, Bz / anb};
            const double pEq = p->p_eq;
            const double div = an[0] * p0[0] + an[1] * p0[1] + an[2] * p0[2];
            const double b = dTime * 4.78941714e+7;
            const double bb[3] = {b * (G[0] * p->dx * ((double)i - 0.5)), b * (G[1] * p->dy * ((double)j - 0.5)),
                                  b * (G[2] * p->dz * ((double)k - 0.5))};
            double dxp = 0, dxm = 0, dyp = 0, dym = 0, dzp = 0, dzm = 0;
            if (p->diffusion == 1) {
                dxp = 2.0 * (D[cxp] * D[c]) / (D[cxp] + D[c] + reg);
                dxm = 2.0 * (D[cxm] * D[c]) / (D[cxm] + D[c] + reg);
                dyp = 2.0 * (D[cyp] * D[c]) / (D[cyp] + D[c] + reg);
                dym = 2.0 * (D[cym] * D[c]) / (D[cym] + D[c] + reg);
                dzp = 2.0 * (D[czp] * D[c]) / (D[czp] + D[c] + reg);
                dzm = 2.0 * (D[czm] * D[c]) / (D[czm] + D[c] + reg);
            }
            double u = 0, v = 0, w = 0;
            if (p->velocity == 1) {
                u = 0.5 * (f->vx[c] + f->vx[cxp]);
                v = 0.5 * (f->vy[c] + f->vy[cyp]);
                w = 0.5 * (f->vz[c] + f->vz[czp]);
            }
            const double* mold[3] = {f->mx, f->my, f->mz};
            double* out[3] = {oX, oY, oZ};
            for (int a = 0; a < 3; a++) {
                const double* m = in[a];
                const double pa = p0[a];
                const double diva = an[a] * div;
                const double rel = dTime * tau1 * (pEq * an[a] - diva) + dTime * tau2 * (diva - pa);
                double vec = 0.0;
                if (p->vector_mult == 1) {
                    if (a == 0) vec = 0.0 - bb[1] * p0[2] + bb[2] * p0[1];
                    if (a == 1) vec = 0.0 + bb[0] * p0[2] - bb[2] * p0[0];
                    if (a == 2) vec = 0.0 - bb[0] * p0[1] + bb[1] * p0[0];
                }
                double dif = 0.0;
                if (p->diffusion == 1)
                    dif = hxx * (dxp * (m[cxp] - pa) - dxm * (pa - m[cxm]))
                        + hyy * (dyp * (m[cyp] - pa) - dym * (pa - m[cym]))
                        + hzz * (dzp * (m[czp] - pa) - dzm * (pa - m[czm]));
                double vel = 0.0;
                if (p->velocity == 1) {
                    if (stage == 0) {
                        const double xm = f->act[cxm] ? m[cxm] : pa, ym = f->act[cym] ? m[cym] : pa;
                        const double zm = f->act[czm] ? m[czm] : pa;
                        vel = 0.0 - u * hx * (pa - xm) - v * hy * (pa - ym) - w * hz * (pa - zm);
                    } else {
                        const double xp = f->act[cxp] ? m[cxp] : pa, yp = f->act[cyp] ? m[cyp] : pa;
                        const double zp = f->act[czp] ? m[czp] : pa;
                        vel = 0.0 - u * hx * (xp - pa) - v * hy * (yp - pa) - w * hz * (zp - pa);
                    }
                }
                if (stage == 0) out[a][c] = pa + rel + vec + dif + vel;
                else out[a][c] = 0.5 * (mold[a][c] + pa + rel + vec + dif + vel);
            }
        }
    }
}

/* OrtTransform (cpp:2536-2550): Rodrigues rotation of one voxel */
static inline void ort(double* x, double* y, double* z, double nx, double ny, double nz, double angle) {
    double c = cos(angle), s = sin(angle);
    double v0x = *x, v0y = *y, v0z = *z;
    double scal = nx * v0x + ny * v0y + nz * v0z;
    *x = v0x * c + nx * (1.0 - c) * scal + s * (ny * v0z - nz * v0y);
    *y = v0y * c + ny * (1.0 - c) * scal + s * (nz * v0x - nx * v0z);
    *z = v0z * c + nz * (1.0 - c) * scal + s * (nx * v0y - ny * v0x);
}

/* AddImpulse (cpp:2552-2608) on the interior pore voxels (ghosts are refreshed
 * by the copy boundary condition right after, as in the reference). */
static void add_impulse(const bto_params* p, ofields_t* f, const bto_pulse* pu) {
    const grid_t* g = &f->g;
    const double nx = pu->axis[0], ny = pu->axis[1], nz = pu->axis[2];
    const double grad = pu->param;
    const double g_ = p->gamma;
    double length = pow(nx * nx + ny * ny + nz * nz, 0.5);
    if (length == 0.0) length = 1.0;
    const double nx0 = nx / length, ny0 = ny / length, nz0 = nz / length;
    const double distance = 10e+12;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= g->nz; k++)
        for (int j = 1; j <= g->ny; j++)
            for (int i = 1; i <= g->nx; i++) {
                size_t c = gidx(g, i, j, k);
                if (f->act[c] != 1) continue;
                double angle;
                if (pu->flag == 1) {
                    angle = grad * g_ * ((i - 1) * p->dx * nx + (j - 1) * p->dy * ny + (k - 1) * p->dz * nz);
                    ort(&f->mx[c], &f->my[c], &f->mz[c], nx0, ny0, nz0, angle);
                } else if (pu->flag == 2) {
                    angle = grad;
                    ort(&f->mx[c], &f->my[c], &f->mz[c], nx, ny, nz, angle);
                } else if (pu->flag == 3) {
                    double effG = pow(nx * nx + ny * ny + nz * nz, 0.5);
                    angle = g_ * effG * pow(pow(((double)i - 1.0 - distance) * p->dx * nx0
                                                + ((double)j - 1.0 - distance) * p->dy * ny0
                                                + ((double)k - 1.0 - distance) * p->dz * nz0, 2), 0.5);
                    ort(&f->mx[c], &f->my[c], &f->mz[c], nx0, ny0, nz0, angle);
                } else if (pu->flag == 4) {
                    angle = 0.0 - g_ * sqrt(pow((i - 0.5) * p->dx * nx - 0.5 * g->nx * p->dx * nx, 2.0)
                                            + pow((j - 0.5) * p->dy * ny - 0.5 * g->ny * p->dy * ny, 2.0)
                                            + pow((k - 0.5) * p->dz * nz - 0.5 * g->nz * p->dz * nz, 2.0));
                    ort(&f->mx[c], &f->my[c], &f->mz[c], nx, ny, nz, angle);
                }
            }
}

/* Physics mode (no reference counterpart): B0 along z, the gradient field
 * B_z(r) = G.r with r = (c + 0.5) * d turns the transverse magnetization by
 * exp(-i * gamma * B_z * frac * dt) (dM/dt = gamma M x B, as the reference's
 * cross product, but integrated exactly); a step applies half of its turn
 * before the explicit relaxation/advection/diffusion update and half after
 * (a symmetric split, second order in dt for the gradient dephasing). */
static void precess_exact(const bto_params* p, ofields_t* f, const double G[3], double frac) {
    const grid_t* g = &f->g;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= g->nz; k++)
        for (int j = 1; j <= g->ny; j++)
            for (int i = 1; i <= g->nx; i++) {
                size_t c = gidx(g, i, j, k);
                if (f->act[c] != 1) continue;
                double bz = G[0] * (((double)i - 0.5) * p->dx) + G[1] * (((double)j - 0.5) * p->dy)
                          + G[2] * (((double)k - 0.5) * p->dz);
                double th = p->gamma * bz * (frac * p->dt);
                double cs = cos(th), sn = sin(th);
                double x = f->mx[c], y = f->my[c];
                f->mx[c] = x * cs + y * sn;
                f->my[c] = y * cs - x * sn;
            }
}

/* OutputX/Y/Z with nComponents == 1: sums over pore voxels inside the
 * buffer-trimmed box. Per-plane partial sums, then added in plane order. */
static long long field_sums(const bto_params* p, const grid_t* g, const char* act,
                            const double* mx, const double* my, const double* mz,
                            double* out, double* scratch) {
    const int k0 = 1 + p->buffer[2], k1 = g->nz + 1 - p->buffer[2];
    const int j0 = 1 + p->buffer[1], j1 = g->ny + 1 - p->buffer[1];
    const int i0 = 1 + p->buffer[0], i1 = g->nx + 1 - p->buffer[0];
    long long count = 0;
    #pragma omp parallel for schedule(static) reduction(+ : count)
    for (int k = k0; k < k1; k++) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int j = j0; j < j1; j++)
            for (int i = i0; i < i1; i++) {
                size_t c = gidx(g, i, j, k);
                if (act[c] == 1) {
                    sx += mx[c]; sy += my[c]; sz += mz[c];
                    count++;
                }
            }
        scratch[3 * k + 0] = sx; scratch[3 * k + 1] = sy; scratch[3 * k + 2] = sz;
    }
    double tx = 0.0, ty = 0.0, tz = 0.0;
    for (int k = k0; k < k1; k++) {
        tx += scratch[3 * k + 0]; ty += scratch[3 * k + 1]; tz += scratch[3 * k + 2];
    }
    out[0] = tx; out[1] = ty; out[2] = tz;
    return count;
}

/* OutputX/Y/Z with two components (cpp:3324-3350): over pore voxels of the
 * trimming box where c1 > 0.8 or c2 > 0.8, sum_1 += M * c1 and sum_2 += M * c2,
 * k outer, j, i inner. out = {x1, y1, z1, x2, y2, z2}. c1, c2 dense. */
static void phase_sums(const bto_params* p, const grid_t* g, const char* act, const double* c1, const double* c2,
                       const double* mx, const double* my, const double* mz, double* out) {
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = 1 + p->buffer[2]; k < g->nz + 1 - p->buffer[2]; k++)
        for (int j = 1 + p->buffer[1]; j < g->ny + 1 - p->buffer[1]; j++)
            for (int i = 1 + p->buffer[0]; i < g->nx + 1 - p->buffer[0]; i++) {
                size_t c = gidx(g, i, j, k);
                if (act[c] != 1) continue;
                size_t q = (size_t)(i - 1) + (size_t)g->nx * ((size_t)(j - 1) + (size_t)g->ny * (k - 1));
                if (!(c1[q] > 0.8 || c2[q] > 0.8)) continue;
                s[0] += mx[c] * c1[q]; s[3] += mx[c] * c2[q];
                s[1] += my[c] * c1[q]; s[4] += my[c] * c2[q];
                s[2] += mz[c] * c1[q]; s[5] += mz[c] * c2[q];
            }
    for (int a = 0; a < 6; a++) out[a] = s[a];
}

static int run_impl(const bto_params* p, const uint8_t* mask,
                    const double* vx, const double* vy, const double* vz,
                    double* mx, double* my, double* mz,
                    long long nsteps, const bto_pulse* pulses, int npulses,
                    const double* grad_wave, const double* t1, const double* t2, const double* diff,
                    const double* c1, const double* c2, double* mt, double* mt6, int threads, int maccormack) {
    if (!p || p->nx <= 0 || p->ny <= 0 || p->nz <= 0 || nsteps < 0) return -1;
    if ((t1 || t2 || diff) && !(t1 && t2 && diff)) return -1;
    if (mt6 && !(c1 && c2)) return -1;
#ifdef _OPENMP
    int saved = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    ofields_t f;
    if (ofields_init(p, mask, vx, vy, vz, mx, my, mz, &f)) return -2;
    if (t1) {
        /* the caller's FillInDiffusinAndTime fields replace the uniform fluid's */
        for (int k = 0; k < p->nz; k++)
            for (int j = 0; j < p->ny; j++)
                for (int i = 0; i < p->nx; i++) {
                    size_t s = (size_t)i + (size_t)p->nx * ((size_t)j + (size_t)p->ny * k);
                    size_t c = gidx(&f.g, i + 1, j + 1, k + 1);
                    f.t1[c] = t1[s]; f.t2[c] = t2[s]; f.D[c] = diff[s];
                }
        bc_copy_d(&f.g, f.D);
    }
    double* scratch = (double*)calloc((size_t)3 * (p->nz + 2), sizeof(double));
    const grid_t* g = &f.g;
    /* MacCormack: the corrector's output (zero in solid and ghosts) */
    double *cx = NULL, *cy = NULL, *cz = NULL;
    if (maccormack) {
        cx = (double*)calloc(g->num, sizeof(double));
        cy = (double*)calloc(g->num, sizeof(double));
        cz = (double*)calloc(g->num, sizeof(double));
    }
    const double t_start = now_s();
    for (long long s = 0; s < nsteps; s++) {
        double G[3] = {p->grad[0], p->grad[1], p->grad[2]};
        if (grad_wave) { G[0] = grad_wave[3 * s]; G[1] = grad_wave[3 * s + 1]; G[2] = grad_wave[3 * s + 2]; }
        if (p->vector_mult == 2) {
            /* physics mode: half the step's precession before the update, half
             * after (a symmetric split), ghosts of the turned field first: copies
             * in the first step (the initial layer), the run's kind afterwards */
            static const int copy_layers[3] = {0, 0, 0};
            const int* bm = s == 0 ? copy_layers : p->boundary;
            precess_exact(p, &f, G, 0.5);
            bc_apply_d(g, f.mx, bm); bc_apply_d(g, f.my, bm); bc_apply_d(g, f.mz, bm);
        }
        if (maccormack) {
            /* predictor into the add arrays (zero in solid), copy ghosts, then
             * the corrector from it into P's partner; M = the corrected field */
            #pragma omp parallel for schedule(static)
            for (size_t q = 0; q < g->num; q++) { f.ax[q] = 0.0; f.ay[q] = 0.0; f.az[q] = 0.0; }
            #pragma omp parallel for schedule(static)
            for (int k = 1; k <= g->nz; k++) mac_plane(p, &f, k, G, 0, f.mx, f.my, f.mz, f.ax, f.ay, f.az);
            bc_apply_d(g, f.ax, p->boundary); bc_apply_d(g, f.ay, p->boundary); bc_apply_d(g, f.az, p->boundary);
            #pragma omp parallel for schedule(static)
            for (int k = 1; k <= g->nz; k++) mac_plane(p, &f, k, G, 1, f.ax, f.ay, f.az, cx, cy, cz);
            #pragma omp parallel for schedule(static)
            for (size_t q = 0; q < g->num; q++) { f.ax[q] = cx[q]; f.ay[q] = cy[q]; f.az[q] = cz[q]; }
        } else {
            #pragma omp parallel for schedule(static)
            for (int k = 1; k <= g->nz; k++) update_plane(p, &f, k, G);
        }
        /* copy the interior back (cpp:3269-3280); solid voxels take the add
         * arrays' untouched value, which is zero */
        #pragma omp parallel for schedule(static)
        for (int k = 1; k <= g->nz; k++)
            for (int j = 1; j <= g->ny; j++) {
                size_t c0 = gidx(g, 1, j, k);
                memcpy(&f.mx[c0], &f.ax[c0], sizeof(double) * g->nx);
                memcpy(&f.my[c0], &f.ay[c0], sizeof(double) * g->nx);
                memcpy(&f.mz[c0], &f.az[c0], sizeof(double) * g->nx);
            }
        if (p->vector_mult == 2) precess_exact(p, &f, G, 0.5);
        for (int q = 0; q < npulses; q++)
            if (pulses[q].step == s) add_impulse(p, &f, &pulses[q]);
        bc_apply_d(g, f.mx, p->boundary); bc_apply_d(g, f.my, p->boundary); bc_apply_d(g, f.mz, p->boundary);
        if (mt) field_sums(p, g, f.act, f.mx, f.my, f.mz, &mt[3 * s], scratch);
        if (mt6) phase_sums(p, g, f.act, c1, c2, f.mx, f.my, f.mz, &mt6[6 * s]);
    }
    g_loop_seconds = now_s() - t_start;
    for (int k = 0; k < p->nz; k++)
        for (int j = 0; j < p->ny; j++)
            for (int i = 0; i < p->nx; i++) {
                size_t s = (size_t)i + (size_t)p->nx * ((size_t)j + (size_t)p->ny * k);
                size_t c = gidx(g, i + 1, j + 1, k + 1);
                mx[s] = f.mx[c]; my[s] = f.my[c]; mz[s] = f.mz[c];
            }
    free(scratch);
    free(cx); free(cy); free(cz);
    ofields_free(&f);
#ifdef _OPENMP
    omp_set_num_threads(saved);
#endif
    return 0;
}

int bto_run_reference(const bto_params* p, const uint8_t* mask,
                      const double* vx, const double* vy, const double* vz,
                      double* mx, double* my, double* mz,
                      long long nsteps, const bto_pulse* pulses, int npulses,
                      const double* grad_wave, double* mt, int threads) {
    return run_impl(p, mask, vx, vy, vz, mx, my, mz, nsteps, pulses, npulses, grad_wave, NULL, NULL, NULL, NULL,
                    NULL, mt, NULL, threads, 0);
}

int bto_run_fields(const bto_params* p, const uint8_t* mask,
                   const double* vx, const double* vy, const double* vz,
                   double* mx, double* my, double* mz,
                   long long nsteps, const bto_pulse* pulses, int npulses, const double* grad_wave,
                   const double* t1, const double* t2, const double* diff,
                   const double* c1, const double* c2, double* mt, double* mt6, int threads) {
    return run_impl(p, mask, vx, vy, vz, mx, my, mz, nsteps, pulses, npulses, grad_wave, t1, t2, diff, c1, c2, mt,
                    mt6, threads, 0);
}

int bto_run_maccormack(const bto_params* p, const uint8_t* mask,
                       const double* vx, const double* vy, const double* vz,
                       double* mx, double* my, double* mz,
                       long long nsteps, const bto_pulse* pulses, int npulses, const double* grad_wave,
                       const double* t1, const double* t2, const double* diff,
                       const double* c1, const double* c2, double* mt, double* mt6, int threads) {
    return run_impl(p, mask, vx, vy, vz, mx, my, mz, nsteps, pulses, npulses, grad_wave, t1, t2, diff, c1, c2, mt,
                    mt6, threads, 1);
}

long long bto_sums(const bto_params* p, const uint8_t* mask,
                   const double* mx, const double* my, const double* mz, double* out) {
    ofields_t f;
    if (ofields_init(p, mask, NULL, NULL, NULL, mx, my, mz, &f)) return -1;
    double* scratch = (double*)calloc((size_t)3 * (p->nz + 2), sizeof(double));
    long long n = field_sums(p, &f.g, f.act, f.mx, f.my, f.mz, out, scratch);
    free(scratch);
    ofields_free(&f);
    return n;
}

void bto_rates(const bto_params* p, const uint8_t* mask, double* tau1, double* tau2) {
    size_t n = (size_t)p->nx * p->ny * p->nz;
    double* z = (double*)calloc(n, sizeof(double));
    ofields_t f;
    if (ofields_init(p, mask, NULL, NULL, NULL, z, z, z, &f)) { free(z); return; }
    for (int k = 0; k < p->nz; k++)
        for (int j = 0; j < p->ny; j++)
            for (int i = 0; i < p->nx; i++) {
                size_t s = (size_t)i + (size_t)p->nx * ((size_t)j + (size_t)p->ny * k);
                size_t c = gidx(&f.g, i + 1, j + 1, k + 1);
                tau1[s] = 1.0 / f.t1[c];
                tau2[s] = 1.0 / f.t2[c];
            }
    ofields_free(&f);
    free(z);
}

int bto_gpu_inputs(const bto_params* p, const uint8_t* mask,
                   const double* vx, const double* vy, const double* vz,
                   const double* mx, const double* my, const double* mz,
                   char* act, double* diff, double* t1, double* t2,
                   double* nf, double* vel, double* magn) {
    if (!p || p->nx <= 0 || p->ny <= 0 || p->nz <= 0) return -1;
    ofields_t f;
    if (ofields_init(p, mask, vx, vy, vz, mx, my, mz, &f)) return -2;
    const grid_t* g = &f.g;
    const size_t num = g->num;
    for (size_t q = 0; q < num; q++) {
        act[q] = f.act[q] ? '1' : '0';
        diff[q] = f.D[q];
        t1[q] = f.t1[q] != 0.0 ? f.t1[q] : BIG;
        t2[q] = f.t2[q] != 0.0 ? f.t2[q] : BIG;
        vel[q] = f.vx[q]; vel[num + q] = f.vy[q]; vel[2 * num + q] = f.vz[q];
        magn[q] = f.mx[q]; magn[num + q] = f.my[q]; magn[2 * num + q] = f.mz[q];
    }
    /* FillInMainField (cpp:1944-1972): G * d * (i - 0.5) over every ghosted index */
    for (int k = 0; k < g->nz + 2; k++)
        for (int j = 0; j < g->ny + 2; j++)
            for (int i = 0; i < g->nx + 2; i++) {
                size_t c = gidx(g, i, j, k);
                nf[c] = p->grad[0] * p->dx * (i - 0.5);
                nf[num + c] = p->grad[1] * p->dy * (j - 0.5);
                nf[2 * num + c] = p->grad[2] * p->dz * (k - 0.5);
            }
    ofields_free(&f);
    return 0;
}
