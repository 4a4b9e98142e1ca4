// The reference's GPU scheme (solve_gpu's ExplicitMakUpgrade, reference
// src/NmrRelaxationSolveKernels.cu:1473-1498) as a compat variant of the step:
// a MacCormack predictor-corrector, two launches per step.
//
//   stage 0 (NMR_predictor_upgrade, cu:637-801): P = M + rates(M), advection
//           with the cell-average velocity and backward differences;
//   stage 1 (NMR_corrector_upgrade, cu:803-967): M' = 0.5 * (M + P + rates(P)),
//           forward differences; then the step's pulses, M(t) and the step
//           counter, as the other step kernels.
//
// rates(): relaxation dTime/T (pEq n - n(n.M)) + dTime/T2 (n(n.M) - M), Euler
// cross product with the gradient noise field, harmonic-mean diffusion with
// the 1e-25 regulariser of those kernels (weights formed on the host), summed
// in the reference's order (FP64 compiled with -fmad=false). In an advective
// difference a solid neighbour holds the voxel's own value: the reference
// writes it there first (a reflection; with several writers its GPU result is
// racy, this is the zero-flux reading). Copy ghosts at the domain faces come
// from index clamping, as in step_kernel; periodic and zero faces
// (bt_config.boundary) from face_ghosts. Same tile and z-march as step_kernel.
#pragma once
#include "bt_step.cuh"

namespace bt {

template <typename T, int STAGE, bool VEL, bool PREC>
__global__ void __launch_bounds__(NTHREADS) mac_kernel(const __grid_constant__ StepParams<T> P) {
    __shared__ T sm[3][TY + 2][TX + 2];
    __shared__ double red[NTHREADS / 32][3];
    __shared__ int last_flag;
    __shared__ PulsePrep pprep;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int x = blockIdx.x * TX + tx;
    const int y = blockIdx.y * TY + ty;
    const unsigned nb = P.nbatch > 1 ? (unsigned)P.nbatch : 1u;
    const int zc = (int)(blockIdx.z % (unsigned)P.zsplit);
    const unsigned b = blockIdx.z / (unsigned)P.zsplit;
    const int z0 = zc * P.zchunk;
    const int z1 = min(nz, z0 + P.zchunk);
    const long long step = __ldcg(&P.ctl->step);
    const StepInfo* si = P.steps + (step < P.nsched ? step : P.nsched) * nb + b;
    // in: the field this stage differentiates (M for the predictor, P for the
    // corrector); orig: M (corrector only)
    const T* in[3] = {P.in[0] + b * P.bstride, P.in[1] + b * P.bstride, P.in[2] + b * P.bstride};
    const T* orig[3] = {nullptr, nullptr, nullptr};
    if constexpr (STAGE == 1)
        for (int c = 0; c < 3; ++c) orig[c] = P.orig[c] + b * P.bstride;
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

    T gdx = 0, gdy = 0, gdz = 0;
    if constexpr (PREC) {
        gdx = (T)(si->grad[0] * P.dxd);
        gdy = (T)(si->grad[1] * P.dyd);
        gdz = (T)(si->grad[2] * P.dzd);
    }
    const int npulse = STAGE == 1 ? si->pulse_count : 0;
    const DevPulse* pulses = P.pulses + si->pulse_first;
    if (npulse) {  // CTA-uniform
        pulse_prep(pprep, pulses, npulse, ty * TX + tx);
        __syncthreads();
    }
    // non-copy domain faces: the predictor reads the field's ghosts, which
    // hold the reference's initial copies in the first step of a run from
    // step 0 (ghost layers are set at the end of each step); the corrector
    // reads the predictor's, set right after the predictor in every step
    const int bcs[3] = {P.bc[0], P.bc[1], P.bc[2]};
    const bool bc_live = (bcs[0] | bcs[1] | bcs[2]) != 0 && (STAGE == 1 || step > 0);
    const bool in_box = x >= P.box[0] && x < P.box[1] && y >= P.box[2] && y < P.box[3];
    Acc<T> accx, accy, accz;

    T cb[3], cc[3], ca[3];
    {
        const int zb = min(max(z0 - 1, 0), nz - 1), zcur = min(z0, nz - 1), za = min(z0 + 1, nz - 1);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cb[c] = in[c][(long long)zb * plane + col];
            cc[c] = in[c][(long long)zcur * plane + col];
            ca[c] = in[c][(long long)za * plane + col];
        }
    }
    T wlo = 0;
    if constexpr (VEL) wlo = P.vz[(long long)min(z0, nz - 1) * plane + col];

    for (int z = z0; z < z1; ++z) {
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
            T o[3] = {0, 0, 0};
            if (cd & CODE_PORE) {
                const int f = cd & 63;
                const long long vox = oz + col;
                const T dtt1 = P.fdtt ? P.fdtt[vox] : P.dtt1[f];
                const T dtt2 = P.fdtt ? P.fdtt[P.fstride + vox] : P.dtt2[f];
                const T p0[3] = {cc[0], cc[1], cc[2]};
                T nbv[3][6];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    nbv[c][0] = sm[c][ty + 1][tx];
                    nbv[c][1] = sm[c][ty + 1][tx + 2];
                    nbv[c][2] = sm[c][ty][tx + 1];
                    nbv[c][3] = sm[c][ty + 2][tx + 1];
                    nbv[c][4] = cb[c];
                    nbv[c][5] = ca[c];
                }
                if (bc_live) {
                    bool open[6] = {x > 0, x < nx - 1, y > 0, y < ny - 1, z > 0, z < nz - 1};
                    const long long far[6] = {oz + (long long)yc * pitch + (nx - 1), oz + (long long)yc * pitch,
                                              oz + (long long)(ny - 1) * pitch + xc, oz + xc,
                                              (long long)(nz - 1) * plane + col, col};
                    face_ghosts<T, SCHEME_REF>(bcs, si, in, far, nbv, open);
                }
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
                const T div = P.an[0] * p0[0] + P.an[1] * p0[1] + P.an[2] * p0[2];
                T bbxb = 0, bbyb = 0, bbzb = 0;
                if constexpr (PREC) {
                    bbxb = P.b * (gdx * ((T)x + (T)0.5));
                    bbyb = P.b * (gdy * ((T)y + (T)0.5));
                    bbzb = P.b * (gdz * ((T)z + (T)0.5));
                }
                T u = 0, v = 0, w = 0;
                if constexpr (VEL) {
                    u = (T)0.5 * (um + up);
                    v = (T)0.5 * (vm + vp);
                    w = (T)0.5 * (wlo + whi);
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T pa = p0[c];
                    const T diva = P.an[c] * div;
                    const T rel = dtt1 * (P.peqn[c] - diva) + dtt2 * (diva - pa);
                    T vec = (T)0.0;
                    if constexpr (PREC) {
                        if (c == 0) vec = (T)0.0 - bbyb * p0[2] + bbzb * p0[1];
                        if (c == 1) vec = (T)0.0 + bbxb * p0[2] - bbzb * p0[0];
                        if (c == 2) vec = (T)0.0 - bbxb * p0[1] + bbyb * p0[0];
                    }
                    T dif = (T)0.0;
                    if (P.diffusion)
                        dif = P.hxx * (dxp * (nbv[c][1] - pa) - dxm * (pa - nbv[c][0])) +
                              P.hyy * (dyp * (nbv[c][3] - pa) - dym * (pa - nbv[c][2])) +
                              P.hzz * (dzp * (nbv[c][5] - pa) - dzm * (pa - nbv[c][4]));
                    T vel = (T)0.0;
                    if constexpr (VEL) {
                        if constexpr (STAGE == 0) {
                            const T xm = (f & 1) ? pa : nbv[c][0], ym = (f & 4) ? pa : nbv[c][2];
                            const T zm = (f & 16) ? pa : nbv[c][4];
                            vel = (T)0.0 - u * P.hx * (pa - xm) - v * P.hy * (pa - ym) - w * P.hz * (pa - zm);
                        } else {
                            const T xp = (f & 2) ? pa : nbv[c][1], yp = (f & 8) ? pa : nbv[c][3];
                            const T zp = (f & 32) ? pa : nbv[c][5];
                            vel = (T)0.0 - u * P.hx * (xp - pa) - v * P.hy * (yp - pa) - w * P.hz * (zp - pa);
                        }
                    }
                    if constexpr (STAGE == 0) o[c] = pa + rel + vec + dif + vel;
                    else o[c] = (T)0.5 * (orig[c][oz + col] + pa + rel + vec + dif + vel);
                }
                if constexpr (STAGE == 1) {
                    if (npulse)
                        apply_pulses<T>(pprep, pulses, npulse, o[0], o[1], o[2], x, y, z, P.dxd, P.dyd, P.dzd,
                                        P.gamma, nx, ny, nz);
                    if (in_box && z >= P.box[4] && z < P.box[5]) {
                        accx.add(o[0]);
                        accy.add(o[1]);
                        accz.add(o[2]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) out[c][oz + col] = o[c];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cb[c] = cc[c];
            cc[c] = ca[c];
            ca[c] = nxt[c];
        }
        if constexpr (VEL) wlo = whi;
    }

    if constexpr (STAGE == 1) {
        double s3[3] = {accx.get(), accy.get(), accz.get()};
        const unsigned local = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (unsigned)zc);
        const unsigned nb_per = gridDim.x * gridDim.y * (unsigned)P.zsplit;
        finish_step<T>(P, step, b, local, nb_per, s3, &red[0][0], &last_flag);
    }
}

template <typename T, int STAGE>
void launch_mac_stage(const StepParams<T>& p, int vel, int prec, dim3 grid, cudaStream_t s) {
    dim3 block(TX, TY);
    if (vel && prec) mac_kernel<T, STAGE, true, true><<<grid, block, 0, s>>>(p);
    else if (vel) mac_kernel<T, STAGE, true, false><<<grid, block, 0, s>>>(p);
    else if (prec) mac_kernel<T, STAGE, false, true><<<grid, block, 0, s>>>(p);
    else mac_kernel<T, STAGE, false, false><<<grid, block, 0, s>>>(p);
}

// both stages of one step: predictor (M -> pred), corrector (pred, M -> out)
template <typename T>
cudaError_t launch_mac_impl(const StepParams<T>& p, T* const pred[3], int vel, int prec, dim3 grid, cudaStream_t s) {
    StepParams<T> a = p;
    for (int c = 0; c < 3; ++c) a.out[c] = pred[c];
    launch_mac_stage<T, 0>(a, vel, prec, grid, s);
    StepParams<T> b = p;
    for (int c = 0; c < 3; ++c) {
        b.orig[c] = p.in[c];
        b.in[c] = pred[c];
    }
    launch_mac_stage<T, 1>(b, vel, prec, grid, s);
    return cudaGetLastError();
}

}  // namespace bt
