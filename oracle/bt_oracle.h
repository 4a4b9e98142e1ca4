/*
 * Oracle for the Bloch–Torrey step: FP64 CPU restatement of the reference
 * solver's explicit update. TEST INFRASTRUCTURE ONLY — used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * Nothing in the product (initializator_gb300/, include/) links or calls it.
 *
 * Layouts (all row-major, x fastest, 0-based interior cells, no ghosts):
 *   mask  [nz][ny][nx]      uint8, 1 = pore ("actCell == '1'"), 0 = solid
 *   state [nz][ny][nx]      double, one array per component
 *   vx    [nz][ny][nx+1]    face velocity, face i is the low face of cell i
 *   vy    [nz][ny+1][nx]
 *   vz    [nz+1][ny][nx]
 * Velocities are already multiplied by VEL_MULT.
 */
#ifndef BT_ORACLE_H
#define BT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;
    double dx, dy, dz, dt;
    double main_field[3];    /* mainField vector (FillInMainField) */
    double gamma;            /* g */
    double grad[3];          /* constGradX/Y/Z, T/m */
    double d_pore;           /* diffusivity of a pore voxel */
    double t1, t2;           /* bulk relaxation times of the fluid */
    double rho1, rho2;       /* surface relaxivities, m/s */
    double p_eq;             /* equilibriumMagnetization */
    int vector_mult;         /* nVectorMult: 1 = reference Euler cross product M x B_noise;
                                2 = exact precession about z by gamma*(G.r)*dt (physics
                                mode, B0 along z; r = (c + 0.5) * d), half of it before
                                the update and half after */
    int velocity;            /* nVelocity */
    int diffusion;           /* nDiffusion */
    int buffer[3];           /* bufferX/Y/Z trimming of the M(t) sums */
    int boundary[3];         /* ghost layers per axis x, y, z after each step (and after the
                                MacCormack predictor): 0 copy (BC_ZeroDer_*, the CPU path's only
                                kind), 1 periodic (BC_Inf_*), 2 zero (BC_Advanced_XM/XP with 0,
                                and the never-written ghosts of pairs the GPU path leaves alone);
                                the first step reads the initial copy ghosts, as the reference's
                                arrays hold them before its first step */
} bto_params;

/* An instantaneous pulse applied after the update of step `step`
 * (AddImpulse flag/param/axis, reference NmrRelaxationSolve.cpp:2552). */
typedef struct {
    long long step;
    int flag;
    int pad;
    double param;
    double axis[3];
} bto_pulse;

/* Advance the field nsteps explicit upwind steps. grad_wave (3*nsteps or NULL)
 * overrides grad per step. mt receives 3*nsteps sums taken after each step
 * (after that step's pulses). threads <= 0 means all cores. Returns 0 on ok. */
int bto_run_reference(const bto_params* p, const uint8_t* mask,
                      const double* vx, const double* vy, const double* vz,
                      double* mx, double* my, double* mz,
                      long long nsteps, const bto_pulse* pulses, int npulses,
                      const double* grad_wave, double* mt, int threads);

/* bto_run_reference with per-voxel coefficients and two-component sums.
 * t1, t2 (s) and diff (m^2/s): dense [nz][ny][nx] arrays that replace what
 * FillInDiffusinAndTime forms for the uniform fluid (all NULL: the fluid of p).
 * c1, c2: dense phase fractions; with mt6 non-NULL, mt6 receives 6*nsteps sums
 * {x1, y1, z1, x2, y2, z2} after each step (OutputX/Y/Z with NCOMP 2,
 * NmrRelaxationSolve.cpp:3324-3350). */
int bto_run_fields(const bto_params* p, const uint8_t* mask,
                   const double* vx, const double* vy, const double* vz,
                   double* mx, double* my, double* mz,
                   long long nsteps, const bto_pulse* pulses, int npulses, const double* grad_wave,
                   const double* t1, const double* t2, const double* diff,
                   const double* c1, const double* c2, double* mt, double* mt6, int threads);

/* bto_run_fields with the reference's GPU scheme (solve_gpu's
 * ExplicitMakUpgrade, NmrRelaxationSolveKernels.cu:1473-1498): MacCormack
 * predictor (backward-difference advection, cu:637-801), copy ghosts,
 * corrector (forward differences, 0.5 * (M + P + terms), cu:803-967) per step.
 * vector_mult 2 is not available in this scheme. */
int bto_run_maccormack(const bto_params* p, const uint8_t* mask,
                       const double* vx, const double* vy, const double* vz,
                       double* mx, double* my, double* mz,
                       long long nsteps, const bto_pulse* pulses, int npulses, const double* grad_wave,
                       const double* t1, const double* t2, const double* diff,
                       const double* c1, const double* c2, double* mt, double* mt6, int threads);

/* The ghosted arrays the reference's GPU path starts from (what InitializeGpu,
 * src/NmrRelaxationSolveKernels.cu:12-88, copies to the device), for running
 * its own kernels: num = (nx+2)(ny+2)(nz+2) cells, x fastest. act: '0'/'1'
 * with the copy ghost layer (BoundaryConditionsForActiveCells); diff, t1, t2:
 * FillInDiffusinAndTime (ghost layer of diff copied; t1, t2 ghosts 1e50, never
 * read); nf: FillInMainField's gradient field G*d*(i - 0.5) (3*num, x y z);
 * vel: ReadVelocity's face velocities (3*num); magn: the field with copy
 * ghosts (3*num). Returns 0 on success. */
int bto_gpu_inputs(const bto_params* p, const uint8_t* mask,
                   const double* vx, const double* vy, const double* vz,
                   const double* mx, const double* my, const double* mz,
                   char* act, double* diff, double* t1, double* t2,
                   double* nf, double* vel, double* magn);

/* Wall time (s) of the stepping loop of the last bto_run_reference call. */
double bto_last_loop_seconds(void);

/* M(t) sums of a field (OutputX/Y/Z). out = {sumx, sumy, sumz}; returns count. */
long long bto_sums(const bto_params* p, const uint8_t* mask,
                   const double* mx, const double* my, const double* mz, double* out);

/* Per-voxel rate 1/T1, 1/T2 exactly as the reference forms tau1/tau2
 * (FillInDiffusinAndTime then 1/relTime). Writes nz*ny*nx each; solid gets 1/1e50. */
void bto_rates(const bto_params* p, const uint8_t* mask, double* tau1, double* tau2);

#ifdef __cplusplus
}
#endif
#endif
