// Fused Bloch–Torrey step kernel (K1) for sm_103a.
//
// One launch = one explicit time step of the whole field plus its M(t) sums:
//   relaxation (T1/T2 with surface rates from the 6 face bits of the voxel
//   code) + precession + first-order upwind advection on face velocities +
//   harmonic-mean 7-point diffusion, then the step's pulses, then the sum of
//   (Mx, My, Mz) over pore voxels of the trimming box.
//
// Reference semantics (soleh00/Initializator):
//   update            src/NmrRelaxationSolve.cpp:3148-3282 (ExplicitSimple)
//   ghost layers      cpp:1664-1754 at one rank: copy -> an out-of-domain
//                     neighbour equals the voxel itself (index clamp here)
//   solid voxels      never updated, stay zero (cpp:3174, 2501-2506)
//   pulses            cpp:2536-2608 (OrtTransform / AddImpulse)
//   M(t)              cpp:3301-3461 (OutputX/Y/Z)
// In double precision (built with -fmad=false) every expression keeps the
// reference's operation order, so the field matches it bit for bit.
//
// Layout: a CTA owns TX x TY columns and marches through its z-chunk. The
// voxel's own column rolls through registers (below / current / above); the
// current plane plus a one-voxel x/y halo sits in shared memory. The sums
// are accumulated per thread (Kahan-compensated in FP32, plain in FP64),
// reduced per CTA in FP64, and the last CTA to finish adds the per-CTA
// partials in a fixed order (deterministic), writes M(t) for the step and
// advances the device step counter, so a captured graph replays any number
// of steps without host involvement.
#pragma once
#include <cmath>
#include "bt_internal.h"

namespace bt {

constexpr int SCHEME_REF = 0;
constexpr int SCHEME_KSPACE = 1;
constexpr int ZCHUNK_MAX = 1024;

template <typename T>
struct Acc;
template <>
struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};
template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double get() const { return s; }
};

// upwind switch v/(v+1e-50) (cpp:3187-3204): exactly 0 for a zero face
// velocity, 1 otherwise (1e-50 underflows in FP32, so FP32 tests v != 0).
__device__ __forceinline__ float upsw(float v) { return v != 0.f ? 1.f : 0.f; }
__device__ __forceinline__ double upsw(double v) { return v / (v + 1.0e-50); }

// OrtTransform (cpp:2536-2550) with the angle's cosine c and sine s given
__device__ __forceinline__ void ort_cs(double& x, double& y, double& z, double nx, double ny, double nz, double c,
                                      double s) {
    double v0x = x, v0y = y, v0z = z;
    double scal = nx * v0x + ny * v0y + nz * v0z;
    x = v0x * c + nx * (1.0 - c) * scal + s * (ny * v0z - nz * v0y);
    y = v0y * c + ny * (1.0 - c) * scal + s * (nz * v0x - nx * v0z);
    z = v0z * c + nz * (1.0 - c) * scal + s * (nx * v0y - ny * v0x);
}

// OrtTransform (cpp:2536-2550) in FP64
__device__ __forceinline__ void ort(double& x, double& y, double& z, double nx, double ny, double nz, double angle) {
    ort_cs(x, y, z, nx, ny, nz, cos(angle), sin(angle));
}

// AddImpulse (cpp:2552-2608) for one voxel; x, y, z are 0-based cell indices
__device__ __forceinline__ void apply_pulse(const DevPulse& pu, double& mx, double& my, double& mz, int x, int y,
                                            int z, double dx, double dy, double dz, double g, int nx, int ny,
                                            int nz) {
    const double ax = pu.axis[0], ay = pu.axis[1], az = pu.axis[2];
    double angle;
    if (pu.flag == 1) {
        angle = pu.param * g * ((double)x * dx * ax + (double)y * dy * ay + (double)z * dz * az);
        ort(mx, my, mz, pu.naxis[0], pu.naxis[1], pu.naxis[2], angle);
    } else if (pu.flag == 2) {
        angle = pu.param;
        ort(mx, my, mz, ax, ay, az, angle);
    } else if (pu.flag == 3) {
        const double distance = 10e+12;
        // pow(pow(X, 2), 0.5) of the reference; glibc's pow returns exactly
        // X*X for exponent 2 and sqrt(Y) for exponent 0.5, which the device
        // reproduces with the correctly rounded forms (the angle is ~1e6 rad,
        // so one ulp of it would move the field by ~1e-10)
        const double X = ((double)(x + 1) - 1.0 - distance) * dx * pu.naxis[0] +
                         ((double)(y + 1) - 1.0 - distance) * dy * pu.naxis[1] +
                         ((double)(z + 1) - 1.0 - distance) * dz * pu.naxis[2];
        angle = g * pu.eff * sqrt(X * X);
        ort(mx, my, mz, pu.naxis[0], pu.naxis[1], pu.naxis[2], angle);
    } else if (pu.flag == 4) {
        const double a = ((double)(x + 1) - 0.5) * dx * ax - 0.5 * nx * dx * ax;
        const double b = ((double)(y + 1) - 0.5) * dy * ay - 0.5 * ny * dy * ay;
        const double c = ((double)(z + 1) - 0.5) * dz * az - 0.5 * nz * dz * az;
        angle = 0.0 - g * sqrt(a * a + b * b + c * c);
        ort(mx, my, mz, ax, ay, az, angle);
    }
}

// A step's pulses, prepared once per CTA. A fixed-angle pulse (flag 2: angle
// param about the axis as given) turns every voxel the same way, so the
// cosine and sine of its angle are formed here once (FP64, by the functions
// the per-voxel form calls, so the FP64 result is unchanged) instead of at
// every voxel. For FP32 fields whose step holds only fixed-angle pulses, rot
// is the product of their matrices (fixed_pulse_then), formed in FP64 and
// applied in FP32.
struct PulsePrep {
    double cs[MAX_PULSES_PER_STEP][2];
    float rot[9];
    int fixed_only;
};

// every thread of the CTA calls it (npulse > 0); a __syncthreads() follows
__device__ __forceinline__ void pulse_prep(PulsePrep& pp, const DevPulse* pulses, int npulse, int tid) {
    if (tid < npulse && tid < MAX_PULSES_PER_STEP && pulses[tid].flag == 2) {
        pp.cs[tid][0] = cos(pulses[tid].param);
        pp.cs[tid][1] = sin(pulses[tid].param);
    }
    if (tid == 0) {
        bool fixed = npulse <= MAX_PULSES_PER_STEP;
        double r[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
        for (int q = 0; fixed && q < npulse; ++q) {
            const DevPulse& pu = pulses[q];
            if (pu.flag != 2) {
                fixed = false;
                break;
            }
            fixed_pulse_then(cos(pu.param), sin(pu.param), pu.axis, r);
        }
        for (int i = 0; i < 9; ++i) pp.rot[i] = (float)r[i];
        pp.fixed_only = fixed ? 1 : 0;
    }
}

// the step's pulses on one voxel's lab-frame (mx, my, mz), x, y, z 0-based
template <typename T>
__device__ __forceinline__ void apply_pulses(const PulsePrep& pp, const DevPulse* pulses, int npulse, T& mx_, T& my_,
                                             T& mz_, int x, int y, int z, double dx, double dy, double dz, double g,
                                             int nx, int ny, int nz) {
    if constexpr (sizeof(T) == 4) {
        if (pp.fixed_only) {
            const float a = mx_, b = my_, c = mz_;
            mx_ = pp.rot[0] * a + pp.rot[1] * b + pp.rot[2] * c;
            my_ = pp.rot[3] * a + pp.rot[4] * b + pp.rot[5] * c;
            mz_ = pp.rot[6] * a + pp.rot[7] * b + pp.rot[8] * c;
            return;
        }
    }
    double mx = mx_, my = my_, mz = mz_;
    for (int q = 0; q < npulse; ++q) {
        const DevPulse& pu = pulses[q];
        if (pu.flag == 2 && q < MAX_PULSES_PER_STEP)
            ort_cs(mx, my, mz, pu.axis[0], pu.axis[1], pu.axis[2], pp.cs[q][0], pp.cs[q][1]);
        else
            apply_pulse(pu, mx, my, mz, x, y, z, dx, dy, dz, g, nx, ny, nz);
    }
    mx_ = (T)mx;
    my_ = (T)my;
    mz_ = (T)mz;
}

// exp(-i * k * (c + 0.5) * d) with the argument formed and reduced in FP64
template <typename T>
__device__ __forceinline__ void lab_phase(double k, int c, double d, T& re, T& im) {
    double a = k * (((double)c + 0.5) * d);
    if constexpr (sizeof(T) == 4) {
        const double two_pi = 6.283185307179586476925286766559;
        a = a - two_pi * rint(a * (1.0 / two_pi));
        float s, cs;
        sincosf((float)a, &s, &cs);
        re = cs;
        im = -s;
    } else {
        double s, cs;
        sincos(a, &s, &cs);
        re = cs;
        im = -s;
    }
}

// Ghost values of the domain faces that are not copy faces (bt_config.boundary):
// zero, or the far edge cell (periodic), in the k frame times the face's wrap
// factor (KSPACE). nb[c][q]: the voxel's neighbours -x +x -y +y -z +z per
// component, holding the copy ghost on domain faces; open[q] becomes true for
// every face given a value here. far[q]: offset of face q's far edge cell.
template <typename T, int SCHEME>
__device__ __forceinline__ void face_ghosts(const int (&bc)[3], const StepInfo* si, const T* const (&in)[3],
                                            const long long (&far)[6], T (&nb)[3][6], bool (&open)[6]) {
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const int kind = bc[q >> 1];
        if (open[q] || kind == BC_COPY) continue;
        T v[3] = {(T)0, (T)0, (T)0};
        if (kind == BC_PERIODIC) {
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c] = in[c][far[q]];
            if constexpr (SCHEME == SCHEME_KSPACE) {
                const T wr = (T)si->wrap[q >> 1][0], wi = (q & 1) ? (T)-si->wrap[q >> 1][1] : (T)si->wrap[q >> 1][1];
                const T re = v[0], im = v[1];
                v[0] = wr * re - wi * im;
                v[1] = wr * im + wi * re;
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) nb[c][q] = v[c];
        open[q] = true;
    }
}

// End of a step, shared by the step kernels: the CTA's sums (FP64) go to its
// slot of the partials (grouped per batch member); the last CTA of the launch
// reduces each member's partials in a fixed order (one warp per member, so
// the result does not depend on scheduling), writes M(t), checks it for
// NaN/Inf and advances the device step counter. red: >= 3 doubles per warp;
// flag: one shared int.
template <typename T>
__device__ __forceinline__ void reduce_partials(const StepParams<T>& P, long long step, unsigned nb_per, double* red);

// the part after each warp's lane 0 has written its 3 sums to red
template <typename T>
__device__ __forceinline__ void finish_step_red(const StepParams<T>& P, long long step, unsigned b, unsigned local,
                                                unsigned nb_per, double* red, int* flag) {
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nwarps = nthreads / 32;
    __syncthreads();
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    if (tid == 0) {
        double t[3] = {0.0, 0.0, 0.0};
        for (int w = 0; w < nwarps; ++w)
#pragma unroll
            for (int c = 0; c < 3; ++c) t[c] += red[w * 3 + c];
#pragma unroll
        for (int c = 0; c < 3; ++c) P.partials[3ull * ((unsigned long long)b * nb_per + local) + c] = t[c];
        __threadfence();
        const unsigned prev = atomicAdd(&P.ctl->ticket, 1u);
        *flag = (prev == nblocks - 1);
    }
    __syncthreads();
    if (!*flag) return;
    __threadfence();
    reduce_partials<T>(P, step, nb_per, red);
}

// all threads of one CTA: step's M(t) (one row per batch member) from the
// per-CTA partials parts, NaN/Inf check; ends with a CTA barrier
template <typename T>
__device__ __forceinline__ void reduce_members(const StepParams<T>& P, const double* parts, long long step,
                                               unsigned nb_per, double* red) {
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthreads / 32;
    const unsigned nb = P.nbatch > 1 ? (unsigned)P.nbatch : 1u;
    const long long slot = step - __ldcg(&P.ctl->mt_base);
    // every thread strides over one member's partials, then a fixed tree
    for (unsigned bb = 0; bb < nb; ++bb) {
        double t[3] = {0.0, 0.0, 0.0};
        for (unsigned q = tid; q < nb_per; q += nthreads)
#pragma unroll
            for (int c = 0; c < 3; ++c) t[c] += __ldcg(&parts[3ull * ((unsigned long long)bb * nb_per + q) + c]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t[c] += __shfl_down_sync(0xffffffffu, t[c], o);
        __syncthreads();  // red is reused
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 3; ++c) red[warp * 3 + c] = t[c];
        __syncthreads();
        if (tid == 0) {
            double u[3] = {0.0, 0.0, 0.0};
            for (int w = 0; w < nwarps; ++w)
#pragma unroll
                for (int c = 0; c < 3; ++c) u[c] += red[w * 3 + c];
            if (slot >= 0 && slot < P.mt_cap) {
#pragma unroll
                for (int c = 0; c < 3; ++c) P.mt[3 * (slot * nb + bb) + c] = u[c];
            } else {
                P.ctl->status |= 1;
            }
            if (!isfinite(u[0]) || !isfinite(u[1]) || !isfinite(u[2])) P.ctl->status |= 4;
        }
    }
    __syncthreads();
}

// the last CTA of a launch (or a finish kernel): M(t) of the step, then the
// step counter
template <typename T>
__device__ __forceinline__ void reduce_partials(const StepParams<T>& P, long long step, unsigned nb_per, double* red) {
    reduce_members<T>(P, P.partials, step, nb_per, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) {
        P.ctl->ticket = 0;
        P.ctl->step = step + 1;
        __threadfence();
    }
}

template <typename T>
__device__ __forceinline__ void finish_step(const StepParams<T>& P, long long step, unsigned b, unsigned local,
                                            unsigned nb_per, double s[3], double* red, int* flag) {
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 3; ++c) red[warp * 3 + c] = s[c];
    finish_step_red<T>(P, step, b, local, nb_per, red, flag);
}

// s + e = a + b exactly (Knuth's TwoSum, FP32)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// FP32 path: the warp-level reduction of the Kahan sums as float-float pairs
// (hi + lo, TwoSum per step) instead of FP64, whose pipe is narrow on this
// part; each warp's pair becomes one FP64 partial at lane 0
__device__ __forceinline__ void finish_step_acc(const StepParams<float>& P, long long step, unsigned b, unsigned local,
                                                unsigned nb_per, const Acc<float> (&acc)[3], double* red, int* flag) {
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float h = acc[c].s, l = -acc[c].c;  // Acc holds s - c
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float bh = __shfl_down_sync(0xffffffffu, h, o), bl = __shfl_down_sync(0xffffffffu, l, o);
            float s, e;
            two_sum(h, bh, s, e);
            e += l + bl;
            h = s + e;
            l = e - (h - s);
        }
        if (lane == 0) red[warp * 3 + c] = (double)h + (double)l;
    }
    finish_step_red<float>(P, step, b, local, nb_per, red, flag);
}

// FP32 fast path: this CTA's M(t) partial only (float-float per warp, FP64
// per CTA, plain store); the next fast step (or the finish kernel closing the
// run) adds the partials, so no CTA waits on a fence or an atomic ticket
__device__ __forceinline__ void cta_partial_acc(const StepParams<float>& P, unsigned b, unsigned local, unsigned nb_per,
                                                const Acc<float> (&acc)[3], double* red) {
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthreads / 32;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float h = acc[c].s, l = -acc[c].c;  // Acc holds s - c
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float bh = __shfl_down_sync(0xffffffffu, h, o), bl = __shfl_down_sync(0xffffffffu, l, o);
            float s, e;
            two_sum(h, bh, s, e);
            e += l + bl;
            h = s + e;
            l = e - (h - s);
        }
        if (lane == 0) reinterpret_cast<float2*>(red)[warp * 3 + c] = make_float2(h, l);
    }
    __syncthreads();
    // the warps' pairs added in warp order, still as float-float (the FP64
    // pipe of this part is a small fraction of the FP32 one), stored in FP64
    if (tid == 0) {
        const float2* pr = reinterpret_cast<const float2*>(red);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float h = pr[c].x, l = pr[c].y;
            for (int w = 1; w < nwarps; ++w) {
                const float2 q = pr[w * 3 + c];
                float s, e;
                two_sum(h, q.x, s, e);
                e += l + q.y;
                h = s + e;
                l = e - (h - s);
            }
            P.partials[3ull * ((unsigned long long)b * nb_per + local) + c] = (double)h + (double)l;
        }
    }
}

// one CTA, closing a run of fast-path steps: the partials of the run's last
// step (P: that step's parameters; nb_per per batch member) -> M(t), NaN/Inf
// check, Ctl::step.
// Launched as a programmatic dependent of the step's grid (or after it in
// plain stream order): it lets the next grid start its CTAs at once (they
// build their tables, then wait for this grid to complete), then waits until
// the step's CTAs have completed and their partials and counter are visible.
template <typename T>
__global__ void __launch_bounds__(256) step_finish_kernel(const __grid_constant__ StepParams<T> P, unsigned nb_per) {
    __shared__ double red[(256 / 32) * 3];
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const long long step = __ldcg(&P.ctl->fstep[1 - P.side]) - 1;
    reduce_partials<T>(P, step, nb_per, red);
}

template <typename T, int SCHEME, bool VEL, bool PREC>
__global__ void __launch_bounds__(NTHREADS) step_kernel(const __grid_constant__ StepParams<T> P) {
    __shared__ T sm[3][TY + 2][TX + 2];
    __shared__ double red[NTHREADS / 32][3];
    __shared__ T exs[TX][2];
    __shared__ T eys[TY][2];
    __shared__ T ezs[SCHEME == SCHEME_KSPACE ? ZCHUNK_MAX : 1][2];
    __shared__ int last_flag;
    __shared__ PulsePrep pprep;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TX + tx;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int x = blockIdx.x * TX + tx;
    const int y = blockIdx.y * TY + ty;
    // blockIdx.z = z-chunk + zsplit * batch member
    const unsigned nb = P.nbatch > 1 ? (unsigned)P.nbatch : 1u;
    const int zc = (int)(blockIdx.z % (unsigned)P.zsplit);
    const unsigned b = blockIdx.z / (unsigned)P.zsplit;
    const int z0 = zc * P.zchunk;
    const int z1 = min(nz, z0 + P.zchunk);
    const long long step = __ldcg(&P.ctl->step);
    const StepInfo* si = P.steps + (step < P.nsched ? step : P.nsched) * nb + b;
    const T* in[3] = {P.in[0] + b * P.bstride, P.in[1] + b * P.bstride, P.in[2] + b * P.bstride};
    T* out[3] = {P.out[0] + b * P.bstride, P.out[1] + b * P.bstride, P.out[2] + b * P.bstride};
    const bool inb = (x < nx) && (y < ny);
    const int xc = min(x, nx - 1), yc = min(y, ny - 1);
    const int pitch = P.pitch;
    const long long plane = P.plane;
    const long long col = (long long)yc * pitch + xc;
    const long long ccol = (long long)yc * P.cpitch + xc;
    const long long cplane = (long long)P.cpitch * ny;
    const long long vxrow = (long long)yc * P.vxpitch + xc;
    const long long vxplane = (long long)ny * P.vxpitch;
    const long long vyplane = (long long)(ny + 1) * pitch;

    // per-step uniform values
    T gdx = 0, gdy = 0, gdz = 0;
    if constexpr (PREC && SCHEME == SCHEME_REF) {
        gdx = (T)(si->grad[0] * P.dxd);
        gdy = (T)(si->grad[1] * P.dyd);
        gdz = (T)(si->grad[2] * P.dzd);
    }
    T ph[6][2];
    if constexpr (SCHEME == SCHEME_KSPACE) {
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            ph[f][0] = (T)si->phase[f][0];
            ph[f][1] = (T)si->phase[f][1];
        }
        // lab-frame phase tables for the frame after this step
        if (ty == 0) lab_phase<T>(si->knext[0], x, P.dxd, exs[tx][0], exs[tx][1]);
        if (ty == 1 && tx < TY) lab_phase<T>(si->knext[1], blockIdx.y * TY + tx, P.dyd, eys[tx][0], eys[tx][1]);
        for (int q = tid; q < z1 - z0; q += NTHREADS) lab_phase<T>(si->knext[2], z0 + q, P.dzd, ezs[q][0], ezs[q][1]);
        __syncthreads();
    }
    const int npulse = si->pulse_count;
    const DevPulse* pulses = P.pulses + si->pulse_first;
    if (npulse) {  // CTA-uniform
        pulse_prep(pprep, pulses, npulse, tid);
        __syncthreads();
    }
    // non-copy domain faces take their own ghosts from the second step on (the
    // first step of a run from step 0 reads the reference's initial copies)
    const int bcs[3] = {P.bc[0], P.bc[1], P.bc[2]};
    const bool bc_live = (bcs[0] | bcs[1] | bcs[2]) != 0 && step > 0;

    const bool in_box = x >= P.box[0] && x < P.box[1] && y >= P.box[2] && y < P.box[3];
    Acc<T> accx, accy, accz;

    // rolling column
    T cb[3], cc[3], ca[3];
    {
        // clamped so that a CTA with an empty chunk (z0 >= nz; the host never
        // makes one) still reads inside the field
        const int zb = min(max(z0 - 1, 0), nz - 1), zcur = min(z0, nz - 1), za = min(z0 + 1, nz - 1);
        const long long ob = (long long)zb * plane + col;
        const long long oc = (long long)zcur * plane + col;
        const long long oa = (long long)za * plane + col;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cb[c] = in[c][ob];
            cc[c] = in[c][oc];
            ca[c] = in[c][oa];
        }
    }
    T wlo = 0;
    if constexpr (VEL) wlo = P.vz[(long long)min(z0, nz - 1) * plane + col];

    for (int z = z0; z < z1; ++z) {
        // prefetch the plane after next for the rolling column
        T nxt[3];
        const long long on = (long long)min(z + 2, nz - 1) * plane + col;
#pragma unroll
        for (int c = 0; c < 3; ++c) nxt[c] = in[c][on];
        const long long oz = (long long)z * plane;
        const uint8_t cd = P.code[(long long)z * cplane + ccol];
        T um = 0, up = 0, vm = 0, vp = 0, whi = 0;
        if constexpr (VEL) {
            um = P.vx[(long long)z * vxplane + vxrow];
            up = P.vx[(long long)z * vxplane + vxrow + 1];
            vm = P.vy[(long long)z * vyplane + col];
            vp = P.vy[(long long)z * vyplane + col + pitch];
            whi = P.vz[(long long)(z + 1) * plane + col];
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 3; ++c) sm[c][ty + 1][tx + 1] = cc[c];
        if (tx == 0) {
            const long long o = oz + (long long)yc * pitch + max(x - 1, 0);
#pragma unroll
            for (int c = 0; c < 3; ++c) sm[c][ty + 1][0] = in[c][o];
        }
        if (tx == TX - 1) {
            const long long o = oz + (long long)yc * pitch + min(x + 1, nx - 1);
#pragma unroll
            for (int c = 0; c < 3; ++c) sm[c][ty + 1][TX + 1] = in[c][o];
        }
        if (ty == 0) {
            const long long o = oz + (long long)max(y - 1, 0) * pitch + xc;
#pragma unroll
            for (int c = 0; c < 3; ++c) sm[c][0][tx + 1] = in[c][o];
        }
        if (ty == TY - 1) {
            const long long o = oz + (long long)min(y + 1, ny - 1) * pitch + xc;
#pragma unroll
            for (int c = 0; c < 3; ++c) sm[c][TY + 1][tx + 1] = in[c][o];
        }
        __syncthreads();

        if (inb) {
            T o0 = 0, o1 = 0, o2 = 0;
            if (cd & CODE_PORE) {
                const int f = cd & 63;
                const long long vox = oz + col;
                T dtt1 = P.fdtt ? P.fdtt[vox] : P.dtt1[f];
                T dtt2 = P.fdtt ? P.fdtt[P.fstride + vox] : P.dtt2[f];
                if (P.pal) {
                    // FP32 per-voxel rates through the rate palette
                    const int id = P.pal_idx[(long long)z * cplane + ccol];
                    dtt1 = (T)P.pal[2 * id];
                    dtt2 = (T)P.pal[2 * id + 1];
                }
                const T px0 = cc[0], py0 = cc[1], pz0 = cc[2];
                // neighbours: -x +x -y +y -z +z, per component
                T nb[3][6];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    nb[c][0] = sm[c][ty + 1][tx];
                    nb[c][1] = sm[c][ty + 1][tx + 2];
                    nb[c][2] = sm[c][ty][tx + 1];
                    nb[c][3] = sm[c][ty + 2][tx + 1];
                    nb[c][4] = cb[c];
                    nb[c][5] = ca[c];
                }
                bool open[6] = {x > 0, x < nx - 1, y > 0, y < ny - 1, z > 0, z < nz - 1};
                if (bc_live) {
                    const long long far[6] = {oz + (long long)yc * pitch + (nx - 1), oz + (long long)yc * pitch,
                                              oz + (long long)(ny - 1) * pitch + xc, oz + xc,
                                              (long long)(nz - 1) * plane + col, col};
                    face_ghosts<T, SCHEME>(bcs, si, in, far, nb, open);
                }
                if constexpr (SCHEME == SCHEME_KSPACE) {
                    // transverse neighbours in the frame of this voxel:
                    // phi_f * m_nb inside the domain and for the ghosts set
                    // above; the voxel itself on a copy face (zero difference)
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const T re = nb[0][q], im = nb[1][q];
                        nb[0][q] = open[q] ? ph[q][0] * re - ph[q][1] * im : px0;
                        nb[1][q] = open[q] ? ph[q][0] * im + ph[q][1] * re : py0;
                    }
                }
                T ax, ay, az;
                if constexpr (SCHEME == SCHEME_REF) {
                    const T div = P.an[0] * px0 + P.an[1] * py0 + P.an[2] * pz0;
                    const T divx = P.an[0] * div, divy = P.an[1] * div, divz = P.an[2] * div;
                    ax = px0 + dtt1 * (P.peqn[0] - divx) + dtt2 * (divx - px0);
                    ay = py0 + dtt1 * (P.peqn[1] - divy) + dtt2 * (divy - py0);
                    az = pz0 + dtt1 * (P.peqn[2] - divz) + dtt2 * (divz - pz0);
                    if constexpr (PREC) {
                        const T bbxb = P.b * (gdx * ((T)x + (T)0.5));
                        const T bbyb = P.b * (gdy * ((T)y + (T)0.5));
                        const T bbzb = P.b * (gdz * ((T)z + (T)0.5));
                        ax += (T)0.0 - bbyb * pz0 + bbzb * py0;
                        ay += (T)0.0 + bbxb * pz0 - bbzb * px0;
                        az += (T)0.0 - bbxb * py0 + bbyb * px0;
                    }
                } else {
                    // B0 along z: the reference relaxation with n = (0, 0, 1)
                    ax = px0 + dtt2 * ((T)0.0 - px0);
                    ay = py0 + dtt2 * ((T)0.0 - py0);
                    az = pz0 + dtt1 * (P.peqn[2] - pz0) + dtt2 * (pz0 - pz0);
                }
                if constexpr (VEL) {
                    const T upp = upsw(up), umm = upsw(um), vpp = upsw(vp), vmm = upsw(vm);
                    const T wpp = upsw(whi), wmm = upsw(wlo);
                    const T u = (T)0.5 * (um + up), v = (T)0.5 * (vm + vp), w = (T)0.5 * (wlo + whi);
                    const T ud = fabs(u), vd = fabs(v), wd = fabs(w);
                    const T hx2 = (T)0.5 * P.hx, hy2 = (T)0.5 * P.hy, hz2 = (T)0.5 * P.hz;
                    const T p0[3] = {px0, py0, pz0};
                    T a[3] = {ax, ay, az};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        a[c] -= hx2 * ((u - ud) * (nb[c][1] - p0[c]) * upp + (u + ud) * (p0[c] - nb[c][0]) * umm) +
                                hy2 * ((v - vd) * (nb[c][3] - p0[c]) * vpp + (v + vd) * (p0[c] - nb[c][2]) * vmm) +
                                hz2 * ((w - wd) * (nb[c][5] - p0[c]) * wpp + (w + wd) * (p0[c] - nb[c][4]) * wmm);
                    }
                    ax = a[0];
                    ay = a[1];
                    az = a[2];
                }
                if (P.diffusion) {
                    T dxm = (f & 1) ? P.dps : P.dpp, dxp = (f & 2) ? P.dps : P.dpp;
                    T dym = (f & 4) ? P.dps : P.dpp, dyp = (f & 8) ? P.dps : P.dpp;
                    T dzm = (f & 16) ? P.dps : P.dpp, dzp = (f & 32) ? P.dps : P.dpp;
                    if (P.fw) {
                        dxm = P.fw[vox];
                        dxp = P.fw[P.fstride + vox];
                        dym = P.fw[2 * P.fstride + vox];
                        dyp = P.fw[3 * P.fstride + vox];
                        dzm = P.fw[4 * P.fstride + vox];
                        dzp = P.fw[5 * P.fstride + vox];
                    }
                    const T p0[3] = {px0, py0, pz0};
                    T a[3] = {ax, ay, az};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        a[c] += P.hxx * (dxp * (nb[c][1] - p0[c]) - dxm * (p0[c] - nb[c][0])) +
                                P.hyy * (dyp * (nb[c][3] - p0[c]) - dym * (p0[c] - nb[c][2])) +
                                P.hzz * (dzp * (nb[c][5] - p0[c]) - dzm * (p0[c] - nb[c][4]));
                    }
                    ax = a[0];
                    ay = a[1];
                    az = a[2];
                }
                T lx = ax, ly = ay;  // lab-frame transverse components
                T er = 1, ei = 0;
                if constexpr (SCHEME == SCHEME_KSPACE) {
                    const T exr = exs[tx][0], exi = exs[tx][1], eyr = eys[ty][0], eyi = eys[ty][1];
                    const T ezr = ezs[z - z0][0], ezi = ezs[z - z0][1];
                    const T xyr = exr * eyr - exi * eyi, xyi = exr * eyi + exi * eyr;
                    er = xyr * ezr - xyi * ezi;
                    ei = xyr * ezi + xyi * ezr;
                    lx = er * ax - ei * ay;
                    ly = er * ay + ei * ax;
                }
                if (npulse) {
                    apply_pulses<T>(pprep, pulses, npulse, lx, ly, az, x, y, z, P.dxd, P.dyd, P.dzd, P.gamma, nx,
                                    ny, nz);
                    if constexpr (SCHEME == SCHEME_KSPACE) {
                        ax = er * lx + ei * ly;  // back to the frame: conj(e) * lab
                        ay = er * ly - ei * lx;
                    } else {
                        ax = lx;
                        ay = ly;
                    }
                }
                o0 = ax;
                o1 = ay;
                o2 = az;
                if (in_box && z >= P.box[4] && z < P.box[5]) {
                    accx.add(lx);
                    accy.add(ly);
                    accz.add(az);
                }
            }
            out[0][oz + col] = o0;
            out[1][oz + col] = o1;
            out[2][oz + col] = o2;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cb[c] = cc[c];
            cc[c] = ca[c];
            ca[c] = nxt[c];
        }
        if constexpr (VEL) wlo = whi;
    }

    // ---- deterministic M(t) reduction ----
    double s3[3] = {accx.get(), accy.get(), accz.get()};
    const unsigned local = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (unsigned)zc);
    const unsigned nb_per = gridDim.x * gridDim.y * (unsigned)P.zsplit;
    finish_step<T>(P, step, b, local, nb_per, s3, &red[0][0], &last_flag);
}

// sums of a field (bt_measure): FP64 per thread, lab frame for a non-zero k
template <typename T>
__global__ void sums_kernel(const __grid_constant__ StepParams<T> P, double kx, double ky, double kz, double* out4) {
    __shared__ double red[NTHREADS / 32][4];
    const int tid = threadIdx.x;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    const long long n = (long long)P.nx * P.ny * P.nz;
    const bool phase = (kx != 0.0 || ky != 0.0 || kz != 0.0);
    for (long long qq = blockIdx.x * (long long)NTHREADS + tid; qq < n; qq += (long long)gridDim.x * NTHREADS) {
        const int x = (int)(qq % P.nx), y = (int)((qq / P.nx) % P.ny), z = (int)(qq / ((long long)P.nx * P.ny));
        if (!(P.code[((long long)z * P.ny + y) * P.cpitch + x] & CODE_PORE)) continue;
        const long long q = ((long long)z * P.ny + y) * P.pitch + x;
        if (x < P.box[0] || x >= P.box[1] || y < P.box[2] || y >= P.box[3] || z < P.box[4] || z >= P.box[5]) continue;
        double a = (double)P.in[0][q], b = (double)P.in[1][q];
        if (phase) {
            double ang = kx * ((x + 0.5) * P.dxd) + ky * ((y + 0.5) * P.dyd) + kz * ((z + 0.5) * P.dzd);
            double sn, cs;
            sincos(ang, &sn, &cs);
            const double ra = cs * a + sn * b, rb = cs * b - sn * a;  // exp(-i ang) * (a + i b)
            a = ra;
            b = rb;
        }
        s[0] += a;
        s[1] += b;
        s[2] += (double)P.in[2][q];
        s[3] += 1.0;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
    if ((tid & 31) == 0)
#pragma unroll
        for (int c = 0; c < 4; ++c) red[tid >> 5][c] = s[c];
    __syncthreads();
    if (tid == 0) {
        double t[4] = {0.0, 0.0, 0.0, 0.0};
        for (int w = 0; w < NTHREADS / 32; ++w)
#pragma unroll
            for (int c = 0; c < 4; ++c) t[c] += red[w][c];
#pragma unroll
        for (int c = 0; c < 4; ++c) P.partials[4ull * blockIdx.x + c] = t[c];
    }
}

// two-component sums (OutputX/Y/Z with NCOMP 2, cpp:3324-3350): per block,
// sum of w1 * M and w2 * M over the newest field (P.out), FP64, in a fixed
// order; w1 / w2 are zero where a voxel is not counted. part6[block][6] =
// {x1, y1, z1, x2, y2, z2}
template <typename T>
__global__ void phase_sums_kernel(const __grid_constant__ StepParams<T> P, const T* w1, const T* w2, double* part6) {
    __shared__ double red[NTHREADS / 32][6];
    const int tid = threadIdx.x;
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const long long n = (long long)P.nx * P.ny * P.nz;
    for (long long qq = blockIdx.x * (long long)NTHREADS + tid; qq < n; qq += (long long)gridDim.x * NTHREADS) {
        const int x = (int)(qq % P.nx), y = (int)((qq / P.nx) % P.ny), z = (int)(qq / ((long long)P.nx * P.ny));
        const long long q = ((long long)z * P.ny + y) * P.pitch + x;
        const double a = (double)w1[q], b = (double)w2[q];
        if (a == 0.0 && b == 0.0) continue;
        const double mx = (double)P.out[0][q], my = (double)P.out[1][q], mz = (double)P.out[2][q];
        s[0] += mx * a;
        s[1] += my * a;
        s[2] += mz * a;
        s[3] += mx * b;
        s[4] += my * b;
        s[5] += mz * b;
    }
#pragma unroll
    for (int c = 0; c < 6; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
    if ((tid & 31) == 0)
#pragma unroll
        for (int c = 0; c < 6; ++c) red[tid >> 5][c] = s[c];
    __syncthreads();
    if (tid == 0) {
        double t[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int w = 0; w < NTHREADS / 32; ++w)
#pragma unroll
            for (int c = 0; c < 6; ++c) t[c] += red[w][c];
#pragma unroll
        for (int c = 0; c < 6; ++c) part6[6ull * blockIdx.x + c] = t[c];
    }
}

// one block: the blocks' partials in a fixed order -> mt6[slot], slot = the
// step just taken (the step kernel has advanced the device counter)
static __global__ void phase_finish_kernel(const Ctl* ctl, const double* part6, int nblocks, double* mt6, long long cap,
                                    int* status) {
    __shared__ double red[NTHREADS / 32][6];
    const int tid = threadIdx.x;
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int q = tid; q < nblocks; q += NTHREADS)
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] += part6[6 * q + c];
#pragma unroll
    for (int c = 0; c < 6; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
    if ((tid & 31) == 0)
#pragma unroll
        for (int c = 0; c < 6; ++c) red[tid >> 5][c] = s[c];
    __syncthreads();
    if (tid == 0) {
        double t[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int w = 0; w < NTHREADS / 32; ++w)
#pragma unroll
            for (int c = 0; c < 6; ++c) t[c] += red[w][c];
        const long long slot = __ldcg(&ctl->step) - 1 - __ldcg(&ctl->mt_base);
        if (slot >= 0 && slot < cap) {
#pragma unroll
            for (int c = 0; c < 6; ++c) mt6[6 * slot + c] = t[c];
        } else {
            atomicOr(status, 1);
        }
    }
}

// frame change of the transverse field: (f0 + i f1) *= exp(sign * i * k.r)
template <typename T>
__global__ void frame_kernel(T* f0, T* f1, const uint8_t* code, int nx, int ny, int nz, int pitch, int cpitch,
                             double kx, double ky, double kz, double dx, double dy, double dz, int sign) {
    const long long n = (long long)nx * ny * nz;
    for (long long qq = blockIdx.x * (long long)blockDim.x + threadIdx.x; qq < n;
         qq += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(qq % nx), y = (int)((qq / nx) % ny), z = (int)(qq / ((long long)nx * ny));
        if (!(code[((long long)z * ny + y) * cpitch + x] & CODE_PORE)) continue;
        const long long q = ((long long)z * ny + y) * pitch + x;
        const double ang = sign * (kx * ((x + 0.5) * dx) + ky * ((y + 0.5) * dy) + kz * ((z + 0.5) * dz));
        double sn, cs;
        sincos(ang, &sn, &cs);
        const double a = (double)f0[q], b = (double)f1[q];
        f0[q] = (T)(cs * a - sn * b);
        f1[q] = (T)(cs * b + sn * a);
    }
}

template <typename T>
cudaError_t launch_step_impl(const StepParams<T>& p, int scheme, int vel, int prec, dim3 grid, cudaStream_t s) {
    dim3 block(TX, TY);
    if (scheme == SCHEME_REF) {
        if (vel && prec) step_kernel<T, SCHEME_REF, true, true><<<grid, block, 0, s>>>(p);
        else if (vel) step_kernel<T, SCHEME_REF, true, false><<<grid, block, 0, s>>>(p);
        else if (prec) step_kernel<T, SCHEME_REF, false, true><<<grid, block, 0, s>>>(p);
        else step_kernel<T, SCHEME_REF, false, false><<<grid, block, 0, s>>>(p);
    } else {
        if (vel) step_kernel<T, SCHEME_KSPACE, true, false><<<grid, block, 0, s>>>(p);
        else step_kernel<T, SCHEME_KSPACE, false, false><<<grid, block, 0, s>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace bt
