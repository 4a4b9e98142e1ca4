// Internal types shared by the step kernels and the host runtime.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace bt {

// z-marching tile: one CTA owns TX x TY columns of a z-chunk.
constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NTHREADS = TX * TY;
// fixed-angle pulses of one step whose cosine and sine the step kernels form
// once per CTA (any further ones in the same step take the per-voxel form)
constexpr int MAX_PULSES_PER_STEP = 8;
// default bound (polls) of the FP32 fast path's plane-ring waits; a healthy
// copy lands in microseconds
constexpr uint32_t RING_WAIT_POLLS = 1u << 20;

// Bits of the per-voxel geometry code (one byte per voxel): bit f (0..5) is
// set when the face neighbour f = -x,+x,-y,+y,-z,+z is an in-domain solid
// voxel; bit 6 is set for a pore voxel. The six face bits index the 64-entry
// relaxation-rate tables (surface relaxation rho/d per solid face).
constexpr uint8_t CODE_PORE = 64;

// KSPACE fast path: axes whose face phase is not identically 1 over the
// schedule (StepParams::phase_axes)
constexpr int PH_NONE = 0;  // no wave vector at any step
constexpr int PH_Z = 1;     // along z only
constexpr int PH_ALL = 2;   // any axis

// ghost layer kinds of a domain-face pair (bt_config.boundary)
constexpr int BC_COPY = 0;
constexpr int BC_PERIODIC = 1;
constexpr int BC_ZERO = 2;

// Per-step schedule record (one per step, read uniformly by every CTA).
struct StepInfo {
    double grad[3];     // gradient during this step, T/m
    double knext[3];    // KSPACE: wave vector after this step (rad/m)
    double phase[6][2]; // KSPACE: face phase factor exp(-i k.(r_nb - r)) for -x,+x,-y,+y,-z,+z
    float phasef[3][2]; // the -x, -y, -z factors rounded to FP32 (the fast path)
    // KSPACE with periodic faces: exp(-i k_a n_a d_a) per axis; the k-frame
    // value of a lower face's ghost is the far edge cell's times this, an
    // upper face's ghost the far edge cell's times its conjugate
    double wrap[3][2];
    float wrapf[3][2];
    int pulse_first;
    int pulse_count;
    // FP32 fast path: when every pulse of the step is fixed-angle (flag 2),
    // rot_ok = 1 and rotf is their product rotation (lab frame, row-major),
    // formed in FP64 and rounded
    int rot_ok;
    float rotf[9];
};

// A fixed-angle pulse (flag 2: angle with cosine c and sine s about the axis
// n as given, OrtTransform's cpp:2536-2550 rotation) acting after the
// rotation r: r <- (c I + (1 - c) n n^T + s [n]x) r
__host__ __device__ inline void fixed_pulse_then(double c, double s, const double n[3], double r[9]) {
    double m[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m[3 * i + j] = (i == j ? c : 0.0) + (1.0 - c) * n[i] * n[j];
    m[1] -= s * n[2];
    m[2] += s * n[1];
    m[3] += s * n[2];
    m[5] -= s * n[0];
    m[6] -= s * n[1];
    m[7] += s * n[0];
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[3 * i + j] = m[3 * i] * r[j] + m[3 * i + 1] * r[3 + j] + m[3 * i + 2] * r[6 + j];
    for (int i = 0; i < 9; ++i) r[i] = t[i];
}

// One pulse, with the reference's normalised axis precomputed on the host.
struct DevPulse {
    int flag;
    int pad;
    double param;
    double axis[3];   // as given (flags 2 and 4 rotate about it)
    double naxis[3];  // axis / |axis| (flags 1 and 3 rotate about it)
    double eff;       // |axis| (flag 3's effective gradient)
};

// Device-side run control: the step index advances inside the kernels so a
// captured CUDA graph can be replayed for any number of steps.
struct Ctl {
    long long step;      // absolute step index of the next launch
    long long mt_base;   // step whose sums go to mt[0]
    unsigned int ticket; // CTAs of the current launch that have finished
    int status;          // 0 ok, 1 = M(t) buffer overflow, 2 = schedule missing
    // FP32 fast path, inside a run of consecutive fast steps: the step index
    // of the next launch on each ping-pong input side (a step on side s reads
    // fstep[s] and writes fstep[1 - s]; step is brought up to date by the
    // finish kernel that closes the run)
    long long fstep[2];
};

// Device layouts are pitched so that every row starts on a 16-byte boundary
// (a TMA requirement): the state, vy and vz use row pitch `pitch` (nx rounded
// up to 4 elements), vx uses `vxpitch` (nx+1 rounded up to 4), the geometry
// code `cpitch` (nx rounded up to 16). Padding columns are never read as data.
template <typename T>
struct StepParams {
    int nx, ny, nz, zchunk;
    int pitch, vxpitch, cpitch;
    int zsplit;                 // z-chunks per field (fast path: per tile column, at most)
    int zlong;                  // fast path: tile columns with zsplit chunks; the rest have zsplit - 1
    int nbatch;                 // fields advanced together (q-sweep); 0 or 1 = one
    long long bstride;          // elements from one batch member's field to the next
    long long plane;            // pitch * ny (state and vz plane stride)
    const T* in[3];
    T* out[3];
    const uint8_t* code;        // [nz][ny][cpitch]
    const T* vx;                // [nz][ny][vxpitch], faces 0..nx
    const T* vy;                // [nz][ny+1][pitch], faces 0..ny
    const T* vz;                // [nz+1][ny][pitch], faces 0..nz
    // reference update constants, formed on the host in FP64 in the
    // reference's operation order, then rounded to T
    T hx, hy, hz, hxx, hyy, hzz;
    T an[3];                    // unit main-field axis
    T peqn[3];                  // pEq * an
    T b;                        // dTime * g
    T dx, dy, dz;
    T dpp, dps;                 // harmonic-mean face diffusivity pore-pore / pore-solid
    T dtt1[64], dtt2[64];       // dTime * (1/T1), dTime * (1/T2) per face code
    int diffusion;
    int bc[3];                  // ghost layer kind per axis (BC_*)
    int phase_axes;             // KSPACE: PH_* of the schedule (the fast path's instance)
    int box[6];                 // M(t) trimming box [x0,x1) [y0,y1) [z0,z1)
    double dxd, dyd, dzd, gamma;  // FP64 copies for pulse angles and k phases
    const StepInfo* steps;      // [(nsched + 1) * nbatch], step-major
    long long nsched;           // steps in the table (entry nsched is the default)
    const DevPulse* pulses;
    Ctl* ctl;
    double* partials;           // [nbatch][CTAs per member][3]
    const double* partials_prev;  // fast path: the other input side's partials (the previous step's)
    int side;                   // ping-pong input side these parameters read
    double* mt;                 // [mt_cap][nbatch][3]
    long long mt_cap;           // steps
    // per-voxel mode (SurfRel*.dat face relaxivities, two-component fluids):
    // when fdtt is set the kernel reads dTime/T1, dTime/T2 from fdtt[0 / fstride
    // + v] and the six face diffusivities (-x +x -y +y -z +z) from
    // fw[f * fstride + v] instead of the code tables; v = z * plane + y * pitch + x
    const T* fdtt;
    const T* fw;
    long long fstride;
    // FP32 per-voxel rates through the rate palette: (dTime/T1, dTime/T2)
    // pairs (256) and each voxel's index ([nz][ny][cpitch] like code; the
    // fast path stages it by TMA); the face weights stay the code table's
    const float* pal;
    const uint8_t* pal_idx;
    const T* orig[3];           // MacCormack corrector: the step's input field M
    // FP32 fast path: polls before a plane-ring wait gives up (RING_WAIT_POLLS
    // unless a test shortens it to see the timeout path run)
    uint32_t wait_polls;
};

// TMA descriptors of the FP32 fast path (one per ping-pong input side)
struct TmaMaps {
    CUtensorMap state;   // 4D {x, y, z, component} over the input field
    CUtensorMap ucell;   // 4D {x, y, z, axis} over the upwind cell velocities
    CUtensorMap code;
    CUtensorMap pal;     // 3D {x, y, z} over the per-voxel rate palette index (uint8)
};

// launchers (bt_step_f32.cu / bt_step_f64.cu)
template <typename T>
cudaError_t launch_step(const StepParams<T>& p, int scheme, int vel, int prec, dim3 grid, cudaStream_t s);
template <typename T>
cudaError_t launch_sums(const StepParams<T>& p, double* out4, cudaStream_t s);
// MacCormack step (predictor into pred, then corrector into p.out)
template <typename T>
cudaError_t launch_mac(const StepParams<T>& p, T* const pred[3], int vel, int prec, dim3 grid, cudaStream_t s);
// two-component weighted sums of the newest field into mt6 (6 per step)
template <typename T>
cudaError_t launch_phase_sums(const StepParams<T>& p, const T* w1, const T* w2, double* part6, int nblocks,
                              double* mt6, long long cap, cudaStream_t s);
// FP32 fast path: TMA-staged plane tiles, 4 voxels per thread, no pulses.
// A run of consecutive fast steps: the first launch has first = true (it
// reads Ctl::step); each later one also reduces its predecessor's partials
// into M(t); launch_tma_finish(last step's parameters) closes the run (the last
// step's M(t), Ctl::step)
// pal: per-voxel rates through the rate palette (p.pal, m.pal); rf: a pulse
// step whose pulses are all fixed-angle (StepInfo::rotf; no palette)
cudaError_t launch_step_tma(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec, bool pal,
                            bool rf, dim3 grid, int tw, bool first, cudaStream_t s);
cudaError_t launch_step_tma64(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec, dim3 grid,
                              bool first, cudaStream_t s);
// the fast path's per-voxel-rate instances (bt_step_tma_pal.cu), both tile widths
cudaError_t launch_step_tma_palette(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec,
                                    dim3 grid, int tw, bool first, cudaStream_t s);
// the fast path's pulse-step instances (bt_step_tma_rf.cu), both tile widths
cudaError_t launch_step_tma_pulse(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec,
                                  dim3 grid, int tw, bool first, cudaStream_t s);
cudaError_t launch_tma_finish(const StepParams<float>& p, dim3 grid, cudaStream_t s);
// upwind cell velocities of the fast path from the face velocities, [axis][z][y][pitch]
cudaError_t launch_cell_velocity(const StepParams<float>& p, float* u, long long comp, cudaStream_t s);
// tile of the fast path: tw = 128 or 64 voxels along x, tile_rows(tw) rows along y
inline int tile_rows(int tw) { return tw == 64 ? 16 : 8; }
template <typename T>
cudaError_t launch_frame(T* f[3], const uint8_t* code, int nx, int ny, int nz, int pitch, int cpitch, double kx,
                         double ky, double kz, double dx, double dy, double dz, int sign, cudaStream_t s);

}  // namespace bt
