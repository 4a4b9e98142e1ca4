/*
 * bt.h — C ABI of the GB300 (sm_103a) Bloch–Torrey magnetization solver.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes. Host
 * buffers belong to the caller, device memory to the library; no pointer
 * escapes. A handle is used by one host thread at a time and owns one CUDA
 * stream; several handles may share a device.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the reference project soleh00/Initializator).
 *
 * Array layouts (x fastest, 0-based interior cells, no ghost layer):
 *   mask  [nz][ny][nx]     uint8, 1 = pore (actCell '1'), 0 = solid
 *   field [nz][ny][nx]     double, one array per component
 *   vx    [nz][ny][nx+1]   face velocities (already times VEL_MULT); face i is
 *   vy    [nz][ny+1][nx]   the low face of cell i, face nx the high face of
 *   vz    [nz+1][ny][nx]   the last cell (Vx/Vy/Vz.dat, cpp:1435-1536)
 */
#ifndef BT_H
#define BT_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference prints and calls exit(), headers/NmrRelaxationSolve.h:14-27) */
#define BT_OK 0
#define BT_E_ARG (-1)      /* bad argument or size */
#define BT_E_CUDA (-2)     /* CUDA runtime error; see bt_last_error */
#define BT_E_NAN (-3)      /* M(t) watchdog: a sum became NaN/Inf */
#define BT_E_STATE (-4)    /* call out of order (e.g. run before geometry) */
#define BT_E_NOMEM (-5)    /* device allocation failed */
#define BT_E_TIMEOUT (-6)  /* a bounded device wait gave up */
#define BT_E_SIZE (-7)     /* grid larger than the allocation-free entry point's limit */

/* precision of the fields and of the per-step arithmetic */
#define BT_F32 0
#define BT_F64 1

/* BT_SCHEME_REFERENCE: the reference's explicit upwind update
 *   (ExplicitSimple, src/NmrRelaxationSolve.cpp:3148-3282): forward Euler
 *   relaxation toward p_eq*n, Euler cross product M x B_noise with
 *   B_noise = (Gx*x, Gy*y, Gz*z), first-order upwind advection on face
 *   velocities, harmonic-mean diffusion; solid voxels stay zero.
 * BT_SCHEME_KSPACE: physics form, B0 along z. The same relaxation,
 *   advection and diffusion stencil, but the gradient precession
 *   exp(-i*gamma*(G.r)*dt) is exact: the transverse field is carried in the
 *   frame of the wave vector k(t) = gamma * int G dt, accumulated in FP64 on
 *   the host, and enters the stencil as per-step face phase factors taken
 *   at the middle of the step (half the step's precession, the stencil, the
 *   other half: second order in dt for the gradient dephasing).
 *   Fields passed in and out are always in the lab frame. */
/* BT_SCHEME_MACCORMACK: the reference's GPU scheme (solve_gpu's
 *   ExplicitMakUpgrade, src/NmrRelaxationSolveKernels.cu:637-967,1473-1498):
 *   predictor with backward-difference advection on the cell-average velocity,
 *   corrector M' = 0.5 (M + P + rates(P)) with forward differences, face
 *   diffusivity 2DaDb/(Da+Db+1e-25); a solid neighbour in an advective
 *   difference holds the voxel's own value (the zero-flux reading of the
 *   reference's reflection writes). Two launches per step, generic kernel. */
#define BT_SCHEME_REFERENCE 0
#define BT_SCHEME_KSPACE 1
#define BT_SCHEME_MACCORMACK 2

/* Ghost layer of a domain-face pair (bt_config.boundary, per axis x, y, z), as
 * the reference's GPU path leaves it after BoundaryConditionsForVectorField_gpu
 * (src/NmrRelaxationSolveKernels.cu:1321-1396) for nBoundary1..6 of
 * Nmr_data.dat (x: 1 and 3, y: 2 and 4, z: 5 and 6):
 *   BT_BC_COPY      both faces 1: the edge cell (BC_ZeroDer_*, cu:969-1000; the
 *                   CPU path's only kind, cpp:1664-1754)
 *   BT_BC_PERIODIC  both faces 3: the far edge cell (BC_Inf_*, cu:1002-1033)
 *   BT_BC_ZERO      x with a face 2: zero (BC_Advanced_XM/XP with 0, cu:1035-1053);
 *                   any other pair, which that routine leaves alone: its ghost
 *                   cells are never written and hold zero
 * In every kind the first step of a run that starts at step 0 reads the
 * field's ghosts as copies of the edge cells, as the reference's arrays hold
 * them before its first step (FillInMagnetization + InitializeGpu); the
 * MacCormack predictor's ghosts follow the kind from the first step on. The
 * face diffusivity of a domain face pairs the edge cell with itself in every
 * kind (BoundaryConditionsForDiffusion copies). */
#define BT_BC_COPY 0
#define BT_BC_PERIODIC 1
#define BT_BC_ZERO 2

typedef struct bt_config {
    int nx, ny, nz;        /* interior cells (Nmr_start.dat: ik, jk, kk) */
    int precision;         /* BT_F32 / BT_F64 */
    int scheme;            /* BT_SCHEME_* */
    int vector_mult;       /* NVECTOR: 1 = precession on (REFERENCE scheme) */
    int velocity;          /* NVELOC: 1 = advection on */
    int diffusion;         /* NDIFFUS: 1 = diffusion on */
    int buffer[3];         /* bufferX/Y/Z: cells trimmed from each side of the M(t) sums */
    int batch;             /* fields advanced together over one geometry (a q-sweep); 0 or 1 = one */
    double dx, dy, dz;     /* voxel edges, m */
    double dt;             /* time step, s */
    double main_field[3];  /* mainField vector (FillInMainField, cpp:1944-1962); its unit vector is n */
    double gamma;          /* gyromagnetic constant g (the reference hard-codes 4.78941714e7) */
    double grad[3];        /* static gradient GRAD_X/Y/Z, T/m (used when no waveform is set) */
    double d_pore;         /* diffusivity of a pore voxel, m^2/s */
    double t1, t2;         /* bulk relaxation times of the fluid, s */
    double rho1, rho2;     /* surface relaxivities, m/s (rate rho/d per solid face) */
    double p_eq;           /* equilibriumMagnetization (cpp:810) */
    int boundary[3];       /* BT_BC_* per axis x, y, z (0 = copy, the default) */
    int reserved;
} bt_config;

/* An instantaneous pulse applied right after the update of step `step`
 * (AddImpulse flag/param/axis, cpp:2552-2608): flag 1 linear-gradient phase
 * param*g*(x*dx*ax + y*dy*ay + z*dz*az) about the normalised axis; flag 2 RF
 * rotation by param about axis; flags 3 and 4 as the reference. The
 * KSPACE scheme accepts flag 2 only (gradients come from the waveform).
 * Several pulses of one step apply in the order given. On FP32 handles a
 * step whose pulses are all flag 2 stays on the TMA fast path (their product
 * rotation, formed in FP64, applied in FP32); other pulse steps, and pulse
 * steps of handles with a rate palette, run on the generic kernel. */
typedef struct bt_pulse {
    long long step;
    int flag;
    int reserved;
    double param;
    double axis[3];
} bt_pulse;

typedef struct bt_handle bt_handle;

/* Allocate a solver on the current CUDA device (replaces InitializeGpu,
 * src/NmrRelaxationSolveKernels.cu:12-88: 27 cudaMalloc of ghosted FP64 grids). */
int bt_create(const bt_config* cfg, bt_handle** out);
int bt_destroy(bt_handle* h);
/* Message of the last failure on this handle ("" when none). */
const char* bt_last_error(const bt_handle* h);

/* Geometry and flow from host buffers (replaces ReadActiveCells +
 * FillInDiffusinAndTime + ReadVelocity + the H2D copies of InitializeGpu,
 * cpp:819-878, 1435-1536, 1756-1893). vx/vy/vz may be NULL when velocity == 0. */
int bt_upload_geometry(bt_handle* h, const uint8_t* mask,
                       const double* vx, const double* vy, const double* vz);

/* Batches (cfg->batch = B > 1): B fields share the geometry and flow and
 * advance together, each with its own gradient waveform (a q-sweep; the
 * reference runs one process per gradient, main.cpp:16-28). Field arrays then
 * hold B consecutive fields per component ([B][nz][ny][nx]), grad_wave is
 * [nwave][B][3], M(t) outputs are [nsteps][B][3] and bt_measure writes 3*B
 * sums; pulses apply to every member. */

/* Whole field in / out in the lab frame (replaces FillInMagnetization,
 * cpp:2472-2517, and the D2H copies of solve_gpu, cu:1193-1201).
 * bt_set_state returns once the host arrays have been read (they may be
 * reused at once); the device copy completes in the handle's stream order,
 * so a following bt_run / bt_get_state sees it. Called while steps queued by
 * bt_run_async still run, it converts the next field on the host meanwhile
 * and its copy follows those steps (FP32 fields up to 2^26 voxels: one
 * staging slot per component, so it does not wait for them). */
int bt_set_state(bt_handle* h, const double* mx, const double* my, const double* mz);
int bt_get_state(bt_handle* h, double* mx, double* my, double* mz);
/* The same through device pointers of the handle's precision (float or
 * double, same layout), for callers whose data is already in HBM. */
int bt_set_state_device(bt_handle* h, const void* mx, const void* my, const void* mz);

/* Pulse list and per-step gradient waveform (replaces Sequence_gpu,
 * cpp:2681-3146, which rotates the whole field on the host). grad_wave holds
 * 3*nwave doubles (T/m) for steps [0, nwave); NULL keeps cfg->grad. */
int bt_set_schedule(bt_handle* h, const bt_pulse* pulses, int npulses,
                    const double* grad_wave, long long nwave);

/* Current step index (0 after bt_create); bt_set_step rewinds or advances the
 * schedule position without touching the field. */
long long bt_step_index(const bt_handle* h);
int bt_set_step(bt_handle* h, long long step);

/* Advance nsteps steps (replaces the solve_gpu time loop, cu:1187-1288, with
 * ExplicitMakUpgrade + Sequence_gpu + BoundaryConditionsForVectorField_gpu +
 * OutputX/Y/Z). mt_out (host, may be NULL) receives 3*nsteps doubles: the
 * M(t) sums (x, y, z) after each step and its pulses. Synchronous. */
int bt_run(bt_handle* h, long long nsteps, double* mt_out);

/* Asynchronous form for timing and pipelines: M(t) stays in the handle's
 * device buffer; bt_read_mt copies the sums of the last bt_run_async. */
int bt_run_async(bt_handle* h, long long nsteps);

/* Per-voxel relaxation and diffusion, for inputs the uniform-fluid
 * coefficients cannot express: SurfRel*.dat face relaxivities and two-component
 * (NCOMP 2) fluids. t1, t2 (s) and diff (m^2/s) are dense [nz][ny][nx] arrays
 * holding what the reference's FillInDiffusinAndTime leaves in relTime.t1,
 * relTime.t2 and diffusion (cpp:1756-1841; solid voxels are ignored). The step
 * then uses dTime*(1/T1), dTime*(1/T2) and the harmonic-mean face diffusivities
 * 2*Da*Db/(Da+Db+1e-50) of ExplicitSimple (cpp:3174-3185), formed here in FP64 in
 * that order (domain faces pair a voxel with itself, as the ghost copy does).
 * All three NULL returns to the coefficients formed from bt_config; a new
 * bt_upload_geometry drops uploaded rates too (upload them after it). FP32
 * handles (not the MacCormack scheme) whose pore voxels all have the
 * configuration's d_pore (solid voxels
 * at most 1e-20 m^2/s) and whose pore voxels' FP32 rate pairs take at most 256
 * values keep them as a rate palette (an 8-bit index per voxel, the code
 * table's face weights) and stay on the TMA fast path; other rates run on
 * the generic kernel, which reads the eight per-voxel fields. */
int bt_upload_rates(bt_handle* h, const double* t1, const double* t2, const double* diff);
/* Per-voxel rates given as a palette (no reference counterpart; the same
 * result as bt_upload_rates with each pore voxel's T1, T2 taken from its entry
 * and diff = d_pore in the pore): n (1..256) entries t1[e], t2[e] (s, host)
 * and `idx`, a dense [nz][ny][nx] uint8 array in device memory holding each
 * pore voxel's entry (< n; solid voxels ignored). FP32 handles, not the
 * MacCormack scheme (BT_E_ARG otherwise); after bt_upload_geometry, which drops
 * it. idx is read on the handle's stream (bt_stream) after the work already
 * queued there, and the copy is complete on return. */
int bt_upload_rate_palette(bt_handle* h, const double* t1, const double* t2, int n, const void* idx);

/* Two-component M(t) (OutputX/Y/Z with NCOMP 2, cpp:3324-3350, written by
 * solve_gpu as "Time; X1; Y1; Z1; X2; Y2; Z2", cu:1211-1217): c1, c2 are the
 * dense [nz][ny][nx] phase fractions (the reference's z1/z2 interpolation of
 * the concentrations). After every step the library sums c1*M and c2*M over
 * pore voxels of the trimming box where c1 > 0.8 or c2 > 0.8. Reference scheme,
 * one field per handle. NULL, NULL switches the sums off. */
int bt_set_phase_weights(bt_handle* h, const double* c1, const double* c2);

/* The two-component sums of the last run: 6*nsteps doubles, per step
 * {x1, y1, z1, x2, y2, z2}. */
int bt_read_mt_phases(bt_handle* h, double* out, long long nsteps);

/* Ragged batch: advance n independent handles (each with its own grid size,
 * geometry and schedule) by nsteps each, asynchronously. Launches are
 * interleaved round robin, one captured graph of steps per handle per round,
 * so small grids on the handles' separate streams run side by side on the
 * GPU; the handles' FP32 fast paths get z-chunks for sharing the GPU (see
 * bt_set_tma_split). Read each handle's M(t) with bt_read_mt. No reference
 * counterpart: the reference runs one sample per process (main.cpp:34-36). */
int bt_run_many(bt_handle* const* hs, int n, long long nsteps);
int bt_read_mt(bt_handle* h, double* mt_out, long long nsteps);
int bt_synchronize(bt_handle* h);
/* The handle's stream as a cudaStream_t (void* keeps this header CUDA-free). */
void* bt_stream(bt_handle* h);

/* M(t) sums of the current field (OutputX/Y/Z, cpp:3301-3461). */
int bt_measure(bt_handle* h, double* sums3);

/* Pick the z-chunking of the FP32 fast path by timing trial_steps steps for
 * each candidate (no reference counterpart: the reference launches one
 * thread per voxel, cu:1475-1476): for one to eight waves of CTAs (and for a
 * batch the first wave counts that give every tile column a chunk), the chunk
 * count that fills exactly that many waves and the even splits around it.
 * The field and step index are restored. *best_chunks (may be NULL) receives
 * the chosen number of chunks per field (as for bt_set_tma_chunks). */
int bt_autotune(bt_handle* h, int trial_steps, int* best_chunks);

/* The FP32 fast path's z-chunking: zsplit chunks per column (<= 0: the
 * default for a handle running alone, about four waves of CTAs). A no-op for
 * handles without the fast path. bt_run_many sets the chunking of its handles
 * for sharing the GPU (about two waves over all of them together); this call
 * (or bt_autotune) sets it back for running alone. */
int bt_set_tma_split(bt_handle* h, int zsplit);
/* The FP32 fast path's z-chunking as a number of chunks per field in total:
 * the tile columns get chunks/tiles or one more (so any count of CTAs, e.g.
 * exactly two waves, can be launched), clamped to at least one chunk per
 * column and chunks of 1..1024 planes; <= 0: the default. A no-op for handles
 * without the fast path. */
int bt_set_tma_chunks(bt_handle* h, int chunks);

/* Failure injection for tests (no reference counterpart): the FP32 fast
 * path's plane-ring waits (mbarrier polls for a plane's TMA copy, and the
 * producer's wait for a free ring slot) give up after `polls` polls, 0 = at
 * once, so that a test sees the bounded-wait path run: every CTA that gives
 * up raises its failure flag, waits (with the full bound) for its own copies
 * in flight and exits, and the run returns BT_E_TIMEOUT; the handle stays
 * usable (bt_set_state, then bt_run). polls < 0 restores the default bound
 * (2^20 polls, far beyond what a healthy copy needs). */
int bt_set_wait_polls(bt_handle* h, long long polls);

/* Device pointers of the current field of batch member `member` (no
 * reference counterpart: the learned closure corrects the field in place).
 * Layout [nz][ny][pitch] in the handle's precision; for the KSPACE scheme the
 * transverse components are in the frame of k at the current step. Valid until
 * the next bt_run / bt_set_state / bt_get_state on the handle; work on them in
 * the handle's stream order (bt_stream). */
int bt_field_device(bt_handle* h, int member, void** mx, void** my, void** mz, int* pitch);

/* Number of kernel launches this handle has issued (a launch inside a replayed
 * CUDA graph counts once per replay). */
long long bt_launch_count(const bt_handle* h);

/* Limits of bt_step_noalloc: its scratch is a fixed array compiled into the
 * library (about 2.4 MB on every device that loads it). */
#define BT_NOALLOC_MAX_VOXELS (1 << 21)   /* nx*ny*nz, e.g. 128^3 */
#define BT_NOALLOC_MAX_BLOCKS 16384       /* CTAs of the step kernel's grid */

/* One step of the REFERENCE-scheme update (the fused kernel bt_run uses for
 * FP64 and for the FP32 steps the fast path does not take) that performs no
 * device allocation. No
 * counterpart in the reference: it exists for callers that may not call
 * cudaMalloc — code running under CUDA stream capture, hosts whose framework
 * has reserved the device's memory for its own pool, plugin hosts that forbid
 * allocations. Every buffer is the caller's device memory, dense layouts as at
 * the top of this file, element type float (BT_F32) or double (BT_F64) per
 * cfg->precision: mask; face velocities (NULL when cfg->velocity == 0); the
 * field in (mx_in, my_in, mz_in) and out (must not alias the inputs); sums
 * receives the three M(t) sums of the new field (3 doubles, device memory).
 * The static gradient cfg->grad applies; no pulses. One field per call:
 * cfg->batch must be 0 or 1, cfg->velocity 0 or 1 and cfg->boundary all
 * BT_BC_COPY (BT_E_ARG otherwise).
 * Asynchronous on `stream` (a cudaStream_t, NULL = legacy default stream).
 * The scratch (run control, schedule record, per-CTA partial sums, geometry
 * code) is one file-scope __device__ array shared by every call on a device
 * and keeping the last call's contents; each call re-initialises it, so calls
 * ordered on one stream are independent, but calls that overlap on the GPU
 * race and must not be issued. The first call on a device (and the first
 * after its context was reset) looks up the array's device address
 * (cudaGetSymbolAddress) and must come before any stream capture: made while
 * `stream` is capturing, it returns BT_E_ARG (message on stderr). Grids
 * above BT_NOALLOC_MAX_VOXELS voxels or
 * BT_NOALLOC_MAX_BLOCKS blocks return BT_E_SIZE (with a message on stderr).
 * A NaN/Inf field shows as non-finite sums (no watchdog status here). */
int bt_step_noalloc(const bt_config* cfg, const uint8_t* mask, const void* vx, const void* vy, const void* vz,
                    const void* mx_in, const void* my_in, const void* mz_in, void* mx_out, void* my_out,
                    void* mz_out, double* sums, void* stream);

/* ---- learned closure: primitives of the 3-D CNN (no reference counterpart) ----
 * A 4-layer net of 3x3x3 convolutions, 16 -> 16 channels, BF16 operands with
 * FP32 accumulation on tcgen05 tensor cores, corrects a 2x-coarse, 4x-dt
 * solve toward the fine one. Activations are channels-last BF16 rows of a
 * zero-padded grid: row q = [sample][z+1][y+1][x+1] of (nx+2, ny+2, nz+2),
 * 16 channels (32 bytes) a row, preceded and followed by
 * bt_conv3d_margin(nx, ny) zero rows; x/out point at the start of the
 * allocation (margin included). FP32 row arrays (pre, outf) have no margin.
 * Weights w[27][16 ci][16 co] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) are packed
 * by bt_conv3d_pack_weights into 27*512-byte forward and data-gradient
 * blocks. All calls are asynchronous on `stream` (a cudaStream_t). */
typedef struct bt_conv3d_args {
    int nb, nx, ny, nz;      /* samples and interior grid */
    int mode;                /* 0: out = GELU(x*w + b) (BF16 rows), pre = x*w + b (FP32 rows)
                                1: outf = x*w + b (FP32 rows)
                                2: out = (x*w) * GELU'(pre) (BF16 rows; data gradient)
                                3: outf = x*w (FP32 rows) */
    int reserved;
    const void* x;           /* BF16 padded rows */
    const void* wpack;       /* 27*512 bytes */
    const float* bias;       /* 16 floats (modes 0, 1) */
    void* out;               /* BF16 padded rows (modes 0, 2); halo rows written as zero */
    float* pre;              /* FP32 rows: written in mode 0 (may be NULL), read in mode 2 */
    float* outf;             /* FP32 rows (modes 1, 3) */
    int* status;             /* device int; bit 8 set when a bounded wait gave up */
} bt_conv3d_args;

long long bt_conv3d_margin(int nx, int ny);
int bt_conv3d(const bt_conv3d_args* a, void* stream);
/* grad[28][16][16]: taps 0..26 = dL/dw[t][ci][co]; row 27, ci 0 = dL/db[co].
 * partial: bt_conv3d_wgrad_scratch(...) floats of device scratch. */
int bt_conv3d_weight_grad(const void* x, const void* dz, int nb, int nx, int ny, int nz, float* partial,
                          float* grad, void* stream);
long long bt_conv3d_wgrad_scratch(int nb, int nx, int ny, int nz);
int bt_conv3d_pack_weights(const float* w, void* wpack_fwd, void* wpack_dgrad, void* stream);
/* AdamW on FP32 parameters (step counts from 1). */
int bt_adamw(float* p, const float* g, float* m, float* v, int n, float lr, float beta1, float beta2, float eps,
             float weight_decay, int step, void* stream);
/* One 128x16x16 tensor-core MMA, D[m][n] = sum_k A[m][k] B[n][k] (A, B
 * row-major BF16, D FP32): checks the descriptor layouts the convolution uses. */
int bt_umma_selftest(const void* a_bf16, const void* b_bf16, float* d, int* status, void* stream);

/* ---- host-only helpers (no GPU needed) ---- */

/* Parameters of the reference's pulse schedules. */
typedef struct bt_sequence_params {
    int n_sequence;          /* NSEQUENCE: 0 FID, 1 CPMG, 2 PFG, 5 inversion, 9, 98, 99 */
    int gpu_variant;         /* 1: Sequence_gpu (cpp:2681-3146), 0: Sequence (cpp:2610-2679) */
    double dt;               /* dTime */
    double time1, time2;     /* TIME1, TIME2 */
    double direction[3];     /* field direction (ReadStart, cpp:783-795) */
    double gradient_pulse;   /* gradientPulse (Nmr_grad.dat line PulseNum[0]) */
    double multiple_gradients[3];  /* multipleGradients (lines PulseNum[0..2]) */
} bt_sequence_params;

/* Replay the reference's schedule over steps [0, nsteps) and list the pulses
 * it applies (time windows [t, t+dt) at currentTime = i*dt, one-shot flags as
 * the reference). Writes at most cap pulses; *count gets the total. */
int bt_sequence_schedule(const bt_sequence_params* sp, long long nsteps,
                         bt_pulse* out, int cap, int* count);

/* Library version string. */
const char* bt_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BT_H */
