// FP32 fast path of the fused step (K1, TMA form) for sm_103a.
//
// Same update, sums and step-counter protocol as step_kernel (bt_step.cuh),
// for steps without pulses:
//   * a CTA owns a 128 x 8 column tile and marches through a z-chunk;
//   * each z-plane of the tile (the three field components with a one-voxel
//     x/y halo, face velocities, geometry code) is fetched by one thread with
//     cp.async.bulk.tensor into a 3-slot shared-memory ring, completion
//     tracked by one mbarrier per slot (expect_tx), so two planes are in
//     flight while the CTA computes the current one;
//   * each thread computes 4 consecutive voxels along x: 128-bit shared
//     loads, 128-bit global stores; the voxel's own z-column (below / current
//     / above) rolls through registers;
//   * the stencil is evaluated as relaxation + sum over the six faces of
//     w_f * (M_f - M_0), w_f folding harmonic-mean diffusion and first-order
//     upwind advection, with w_f = 0 on domain faces (copy ghosts give a zero
//     difference in the reference, cpp:1664-1754) — FP32 only; the FP64 path
//     keeps the reference's exact operation order in step_kernel.
// Out-of-range TMA boxes (halo beyond the domain, plane -1 or nz) are
// zero-filled and never used as data.
// Every mbarrier wait is bounded; on timeout the CTA records status bit 8,
// drains its copies (bounded) and returns without touching the step counter.
#pragma once
#include "bt_step.cuh"

namespace bt {

namespace tma {

constexpr int QX = 4;               // voxels per thread along x
constexpr int TW = TMA_TX;          // 128
constexpr int TH = TMA_TY;          // 8
constexpr int NT = 32 * TH;         // 256 threads, one warp per row
constexpr int NSTAGE = 3;
constexpr int SW = TW + 8;          // state tile width: x0-4 .. x0+TW+3
constexpr int SH = TH + 2;          // state tile height: y0-1 .. y0+TH
constexpr int VXW = TW + 4;         // vx faces x0 .. x0+TW+3 (TW+1 used)
constexpr int OFF_STATE = 0;
constexpr int SZ_STATE = 3 * SH * SW * 4;                   // 16320
constexpr int OFF_VX = 16384;
constexpr int SZ_VX = TH * VXW * 4;                         // 4224
constexpr int OFF_VY = OFF_VX + SZ_VX;                      // 20608
constexpr int SZ_VY = (TH + 1) * TW * 4;                    // 4608
constexpr int OFF_VZ = OFF_VY + SZ_VY;                      // 25216
constexpr int SZ_VZ = TH * TW * 4;                          // 4096
constexpr int OFF_CODE = OFF_VZ + SZ_VZ;                    // 29312
constexpr int SZ_CODE = TH * TW;                            // 1024
constexpr int STAGE = OFF_CODE + SZ_CODE;                   // 30336
constexpr int OFF_AUX = NSTAGE * STAGE;                     // tables, barriers, reduction
constexpr int SMEM = OFF_AUX + 2048 + 8 * ZCHUNK_MAX + 128;  // + 128 for the base alignment
static_assert(OFF_VX % 128 == 0 && OFF_VY % 128 == 0 && OFF_VZ % 128 == 0 && OFF_CODE % 128 == 0, "align");
static_assert(STAGE % 128 == 0, "align");
constexpr uint32_t WAIT_LIMIT = 1u << 20;  // polls; a healthy copy lands in microseconds

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(sa(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false after WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(sa(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(sa(bar))
        : "memory");
}

}  // namespace tma

template <int SCHEME, bool VEL, bool PREC>
__global__ void __launch_bounds__(tma::NT, 2)
    step_tma_kernel(const __grid_constant__ StepParams<float> P, const __grid_constant__ TmaMaps M) {
    using namespace tma;
    // TMA destinations must sit on 128-byte boundaries: align the dynamic
    // shared-memory base explicitly (the launch reserves 128 spare bytes)
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((128u - (sa(smem_raw) & 127u)) & 127u);
    float* s_dtt1 = reinterpret_cast<float*>(smem + OFF_AUX);           // 64
    float* s_dtt2 = s_dtt1 + 64;                                        // 64
    float2* s_ex = reinterpret_cast<float2*>(s_dtt2 + 64);              // TW
    float2* s_ey = s_ex + TW;                                           // TH
    // aux layout (bytes from OFF_AUX): dtt1 0..255, dtt2 256..511, ex 512..1535,
    // ey 1536..1599, barriers 1600..1623, flags 1664..1671, red 1728..1919, ez 2048..
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + OFF_AUX + 1600);  // NSTAGE
    int* s_flags = reinterpret_cast<int*>(smem + OFF_AUX + 1664);       // abort, last
    double* red = reinterpret_cast<double*>(smem + OFF_AUX + 1728);     // [TH][3]
    float2* s_ez = reinterpret_cast<float2*>(smem + OFF_AUX + 2048);    // ZCHUNK_MAX

    const int tid = threadIdx.x;
    const int lane = tid & 31, w = tid >> 5;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    // blockIdx.x walks the z-chunks of one tile, so neighbouring chunks (which
    // share their boundary planes) run side by side and meet in L2
    const int zc = blockIdx.x;
    const int x0 = blockIdx.y * TW, y0 = blockIdx.z * TH;
    const int z0 = zc * P.zchunk;
    const int z1 = min(nz, z0 + P.zchunk);
    const long long step = __ldcg(&P.ctl->step);
    const StepInfo* si = P.steps + (step < P.nsched ? step : P.nsched);
    const int xb = x0 + QX * lane;        // first of this thread's 4 voxels
    const int y = y0 + w;

    uint32_t txbytes = SZ_STATE + SZ_CODE;
    if constexpr (VEL) txbytes += SZ_VX + SZ_VY + SZ_VZ;
    auto issue = [&](int slot, int plane) {
        uint64_t* bar = &bars[slot];
        unsigned char* base = smem + slot * STAGE;
        mbar_expect_tx(bar, txbytes);
        tma_load_4d(base + OFF_STATE, &M.state, bar, x0 - 4, y0 - 1, plane, 0);
        if constexpr (VEL) {
            tma_load_3d(base + OFF_VX, &M.vx, bar, x0, y0, plane);
            tma_load_3d(base + OFF_VY, &M.vy, bar, x0, y0, plane);
            tma_load_3d(base + OFF_VZ, &M.vz, bar, x0, y0, plane);
        }
        tma_load_3d(base + OFF_CODE, &M.code, bar, x0, y0, plane);
    };
    // the host never makes an empty chunk; a CTA that still gets one issues
    // no copy, waits on nothing and contributes zero sums
    const bool empty = z1 <= z0;
    const int nplanes = empty ? 0 : z1 - z0 + 2;  // z0-1 .. z1
    int issued[NSTAGE] = {0, 0, 0};              // copies issued per slot (thread 0)
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
        s_flags[0] = 0;
        for (int q = 0; q < NSTAGE && q < nplanes; ++q) {
            issue(q, z0 - 1 + q);
            issued[q]++;
        }
    }
    // per-CTA tables
    if (tid < 64) {
        s_dtt1[tid] = P.dtt1[tid];
        s_dtt2[tid] = P.dtt2[tid];
    }
    if constexpr (SCHEME == SCHEME_KSPACE) {
        if (tid < TW) lab_phase<float>(si->knext[0], x0 + tid, P.dxd, s_ex[tid].x, s_ex[tid].y);
        if (tid >= TW && tid < TW + TH) lab_phase<float>(si->knext[1], y0 + tid - TW, P.dyd, s_ey[tid - TW].x, s_ey[tid - TW].y);
        for (int q = tid; q < z1 - z0; q += NT) lab_phase<float>(si->knext[2], z0 + q, P.dzd, s_ez[q].x, s_ez[q].y);
    }
    __syncthreads();

    // per-step uniforms
    float gdx = 0.f, gdy = 0.f, gdz = 0.f;
    if constexpr (PREC && SCHEME == SCHEME_REF) {
        gdx = (float)(si->grad[0] * P.dxd);
        gdy = (float)(si->grad[1] * P.dyd);
        gdz = (float)(si->grad[2] * P.dzd);
    }
    float ph[6][2];
    if constexpr (SCHEME == SCHEME_KSPACE) {
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            ph[f][0] = (float)si->phase[f][0];
            ph[f][1] = (float)si->phase[f][1];
        }
    }
    const float kpp_x = P.hxx * P.dpp, kps_x = P.hxx * P.dps;
    const float kpp_y = P.hyy * P.dpp, kps_y = P.hyy * P.dps;
    const float kpp_z = P.hzz * P.dpp, kps_z = P.hzz * P.dps;
    const float dmul = P.diffusion ? 1.f : 0.f;
    const float hx2 = 0.5f * P.hx, hy2 = 0.5f * P.hy, hz2 = 0.5f * P.hz;
    const bool row_in = y < ny && y >= P.box[2] && y < P.box[3];

    Acc<float> acc[3];
    float below[3][QX], cur[3][QX], above[3][QX];
    float vzlo[QX] = {0.f, 0.f, 0.f, 0.f}, vzhi[QX] = {0.f, 0.f, 0.f, 0.f};

    auto own = [&](int slot, float (&dst)[3][QX]) {
        const float* st = reinterpret_cast<const float*>(smem + slot * STAGE + OFF_STATE);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float4 v = *reinterpret_cast<const float4*>(st + (c * SH + w + 1) * SW + 4 + QX * lane);
            dst[c][0] = v.x; dst[c][1] = v.y; dst[c][2] = v.z; dst[c][3] = v.w;
        }
    };
    bool ok = true;
    uint32_t uses[NSTAGE] = {0u, 0u, 0u};
    auto wait_slot = [&](int q) {  // q: plane index relative to z0-1
        const int slot = q % NSTAGE;
        if (!mbar_wait(&bars[slot], uses[slot] & 1u)) ok = false;
        uses[slot]++;
        return slot;
    };

    // prologue: below (plane z0-1) and cur (plane z0)
    if (!empty) {
        const int sb = wait_slot(0);
        own(sb, below);
        const int sc = wait_slot(1);
        own(sc, cur);
        if constexpr (VEL) {
            const float4 v = *reinterpret_cast<const float4*>(smem + sc * STAGE + OFF_VZ + 4 * (w * TW + QX * lane));
            vzlo[0] = v.x; vzlo[1] = v.y; vzlo[2] = v.z; vzlo[3] = v.w;
        }
        if (!ok) s_flags[0] = 1;
        __syncthreads();
        if (s_flags[0]) goto abort;
        if (tid == 0 && nplanes > NSTAGE) {
            fence_proxy_async();
            issue(sb, z0 - 1 + NSTAGE);
            issued[sb]++;
        }
    }

    for (int z = z0; z < z1; ++z) {
        const int q = z - (z0 - 1);
        const int sc = q % NSTAGE;
        const int sa_ = wait_slot(q + 1);
        own(sa_, above);
        if constexpr (VEL) {
            const float4 v = *reinterpret_cast<const float4*>(smem + sa_ * STAGE + OFF_VZ + 4 * (w * TW + QX * lane));
            vzhi[0] = v.x; vzhi[1] = v.y; vzhi[2] = v.z; vzhi[3] = v.w;
        }
        if (!ok) s_flags[0] = 1;
        const unsigned char* base = smem + sc * STAGE;
        const float* st = reinterpret_cast<const float*>(base + OFF_STATE);
        // neighbours in the plane
        float xm[3][QX], xp[3][QX], ym[3][QX], yp[3][QX];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* row = st + (c * SH + w + 1) * SW + 4 + QX * lane;
            const float4 a = *reinterpret_cast<const float4*>(row - SW);
            const float4 b = *reinterpret_cast<const float4*>(row + SW);
            ym[c][0] = a.x; ym[c][1] = a.y; ym[c][2] = a.z; ym[c][3] = a.w;
            yp[c][0] = b.x; yp[c][1] = b.y; yp[c][2] = b.z; yp[c][3] = b.w;
            xm[c][0] = row[-1];
            xp[c][3] = row[4];
#pragma unroll
            for (int i = 1; i < QX; ++i) xm[c][i] = cur[c][i - 1];
#pragma unroll
            for (int i = 0; i < QX - 1; ++i) xp[c][i] = cur[c][i + 1];
        }
        const uint32_t code4 = *reinterpret_cast<const uint32_t*>(base + OFF_CODE + w * TW + QX * lane);
        float vxf[QX + 1] = {0.f, 0.f, 0.f, 0.f, 0.f}, vyl[QX] = {0.f, 0.f, 0.f, 0.f}, vyh[QX] = {0.f, 0.f, 0.f, 0.f};
        if constexpr (VEL) {
            const float* vxr = reinterpret_cast<const float*>(base + OFF_VX) + w * VXW + QX * lane;
            const float4 a = *reinterpret_cast<const float4*>(vxr);
            vxf[0] = a.x; vxf[1] = a.y; vxf[2] = a.z; vxf[3] = a.w; vxf[4] = vxr[4];
            const float* vyr = reinterpret_cast<const float*>(base + OFF_VY) + w * TW + QX * lane;
            const float4 b = *reinterpret_cast<const float4*>(vyr);
            const float4 c = *reinterpret_cast<const float4*>(vyr + TW);
            vyl[0] = b.x; vyl[1] = b.y; vyl[2] = b.z; vyl[3] = b.w;
            vyh[0] = c.x; vyh[1] = c.y; vyh[2] = c.z; vyh[3] = c.w;
        }
        float2 ez = make_float2(1.f, 0.f);
        if constexpr (SCHEME == SCHEME_KSPACE) ez = s_ez[z - z0];
        const bool zin = z >= P.box[4] && z < P.box[5];
        float o[3][QX];
#pragma unroll
        for (int i = 0; i < QX; ++i) {
            const int x = xb + i;
            const uint32_t cd = (code4 >> (8 * i)) & 0xffu;
            o[0][i] = 0.f; o[1][i] = 0.f; o[2][i] = 0.f;
            if (!(cd & CODE_PORE) || x >= nx || y >= ny) continue;
            const int f = cd & 63;
            const float dtt1 = s_dtt1[f], dtt2 = s_dtt2[f];
            // face weights: coefficient of (M_face - M_0)
            float wxm = dmul * ((f & 1) ? kps_x : kpp_x), wxp = dmul * ((f & 2) ? kps_x : kpp_x);
            float wym = dmul * ((f & 4) ? kps_y : kpp_y), wyp = dmul * ((f & 8) ? kps_y : kpp_y);
            float wzm = dmul * ((f & 16) ? kps_z : kpp_z), wzp = dmul * ((f & 32) ? kps_z : kpp_z);
            if constexpr (VEL) {
                const float um = vxf[i], up = vxf[i + 1], vm = vyl[i], vp = vyh[i], wm = vzlo[i], wp = vzhi[i];
                const float u = 0.5f * (um + up), v = 0.5f * (vm + vp), ww = 0.5f * (wm + wp);
                const float ud = fabsf(u), vd = fabsf(v), wd = fabsf(ww);
                wxp -= hx2 * (u - ud) * upsw(up);
                wxm += hx2 * (u + ud) * upsw(um);
                wyp -= hy2 * (v - vd) * upsw(vp);
                wym += hy2 * (v + vd) * upsw(vm);
                wzp -= hz2 * (ww - wd) * upsw(wp);
                wzm += hz2 * (ww + wd) * upsw(wm);
            }
            // domain faces: the copy ghost gives a zero difference
            if (x == 0) wxm = 0.f;
            if (x == nx - 1) wxp = 0.f;
            if (y == 0) wym = 0.f;
            if (y == ny - 1) wyp = 0.f;
            if (z == 0) wzm = 0.f;
            if (z == nz - 1) wzp = 0.f;
            const float wsum = ((wxm + wxp) + (wym + wyp)) + (wzm + wzp);
            const float px0 = cur[0][i], py0 = cur[1][i], pz0 = cur[2][i];
            float ax, ay, az;
            if constexpr (SCHEME == SCHEME_REF) {
                const float div = P.an[0] * px0 + P.an[1] * py0 + P.an[2] * pz0;
                const float divx = P.an[0] * div, divy = P.an[1] * div, divz = P.an[2] * div;
                ax = px0 + dtt1 * (P.peqn[0] - divx) + dtt2 * (divx - px0);
                ay = py0 + dtt1 * (P.peqn[1] - divy) + dtt2 * (divy - py0);
                az = pz0 + dtt1 * (P.peqn[2] - divz) + dtt2 * (divz - pz0);
                if constexpr (PREC) {
                    const float bbxb = P.b * (gdx * ((float)x + 0.5f));
                    const float bbyb = P.b * (gdy * ((float)y + 0.5f));
                    const float bbzb = P.b * (gdz * ((float)z + 0.5f));
                    ax += bbzb * py0 - bbyb * pz0;
                    ay += bbxb * pz0 - bbzb * px0;
                    az += bbyb * px0 - bbxb * py0;
                }
                ax += wxm * xm[0][i] + wxp * xp[0][i] + wym * ym[0][i] + wyp * yp[0][i] + wzm * below[0][i] +
                      wzp * above[0][i] - wsum * px0;
                ay += wxm * xm[1][i] + wxp * xp[1][i] + wym * ym[1][i] + wyp * yp[1][i] + wzm * below[1][i] +
                      wzp * above[1][i] - wsum * py0;
            } else {
                ax = px0 - dtt2 * px0;
                ay = py0 - dtt2 * py0;
                az = pz0 + dtt1 * (P.peqn[2] - pz0);
                // transverse: sum_f w_f (phi_f m_f) - W m_0, phi_f the face phase of this step
                const float nbr[6] = {xm[0][i], xp[0][i], ym[0][i], yp[0][i], below[0][i], above[0][i]};
                const float nbi[6] = {xm[1][i], xp[1][i], ym[1][i], yp[1][i], below[1][i], above[1][i]};
                const float wf[6] = {wxm, wxp, wym, wyp, wzm, wzp};
                float sr = -wsum * px0, si_ = -wsum * py0;
#pragma unroll
                for (int f6 = 0; f6 < 6; ++f6) {
                    const float cr = wf[f6] * ph[f6][0], ci = wf[f6] * ph[f6][1];
                    sr += cr * nbr[f6] - ci * nbi[f6];
                    si_ += cr * nbi[f6] + ci * nbr[f6];
                }
                ax += sr;
                ay += si_;
            }
            az += wxm * xm[2][i] + wxp * xp[2][i] + wym * ym[2][i] + wyp * yp[2][i] + wzm * below[2][i] +
                  wzp * above[2][i] - wsum * pz0;
            o[0][i] = ax;
            o[1][i] = ay;
            o[2][i] = az;
            if (row_in && zin && x >= P.box[0] && x < P.box[1]) {
                if constexpr (SCHEME == SCHEME_KSPACE) {
                    const float2 ex = s_ex[QX * lane + i], ey = s_ey[w];
                    const float xyr = ex.x * ey.x - ex.y * ey.y, xyi = ex.x * ey.y + ex.y * ey.x;
                    const float er = xyr * ez.x - xyi * ez.y, ei = xyr * ez.y + xyi * ez.x;
                    acc[0].add(er * ax - ei * ay);
                    acc[1].add(er * ay + ei * ax);
                } else {
                    acc[0].add(ax);
                    acc[1].add(ay);
                }
                acc[2].add(az);
            }
        }
        if (y < ny && xb < nx) {
            const long long off = (long long)z * P.plane + (long long)y * P.pitch + xb;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                *reinterpret_cast<float4*>(P.out[c] + off) = make_float4(o[c][0], o[c][1], o[c][2], o[c][3]);
        }
        __syncthreads();  // every thread is done with slot sc
        if (s_flags[0]) goto abort;
        if (tid == 0 && q + NSTAGE < nplanes) {
            fence_proxy_async();
            issue(sc, z0 - 1 + q + NSTAGE);
            issued[sc]++;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int i = 0; i < QX; ++i) {
                below[c][i] = cur[c][i];
                cur[c][i] = above[c][i];
            }
#pragma unroll
        for (int i = 0; i < QX; ++i) vzlo[i] = vzhi[i];
    }

    // ---- deterministic M(t) reduction (as step_kernel) ----
    {
        double s3[3] = {acc[0].get(), acc[1].get(), acc[2].get()};
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s3[c] += __shfl_down_sync(0xffffffffu, s3[c], o);
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 3; ++c) red[w * 3 + c] = s3[c];
        __syncthreads();
        const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
        const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        if (tid == 0) {
            double t[3] = {0.0, 0.0, 0.0};
            for (int ww = 0; ww < TH; ++ww)
#pragma unroll
                for (int c = 0; c < 3; ++c) t[c] += red[ww * 3 + c];
#pragma unroll
            for (int c = 0; c < 3; ++c) P.partials[3ull * bid + c] = t[c];
            __threadfence();
            const unsigned prev = atomicAdd(&P.ctl->ticket, 1u);
            s_flags[1] = (prev == nblocks - 1);
        }
        __syncthreads();
        if (!s_flags[1]) return;
        __threadfence();
        double t[3] = {0.0, 0.0, 0.0};
        for (unsigned qb = tid; qb < nblocks; qb += NT)
#pragma unroll
            for (int c = 0; c < 3; ++c) t[c] += __ldcg(&P.partials[3ull * qb + c]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t[c] += __shfl_down_sync(0xffffffffu, t[c], o);
        __syncthreads();
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 3; ++c) red[w * 3 + c] = t[c];
        __syncthreads();
        if (tid == 0) {
            double u[3] = {0.0, 0.0, 0.0};
            for (int ww = 0; ww < TH; ++ww)
#pragma unroll
                for (int c = 0; c < 3; ++c) u[c] += red[ww * 3 + c];
            const long long slot = step - __ldcg(&P.ctl->mt_base);
            if (slot >= 0 && slot < P.mt_cap) {
#pragma unroll
                for (int c = 0; c < 3; ++c) P.mt[3 * slot + c] = u[c];
            } else {
                P.ctl->status |= 1;
            }
            if (!isfinite(u[0]) || !isfinite(u[1]) || !isfinite(u[2])) P.ctl->status |= 4;
            P.ctl->ticket = 0;
            P.ctl->step = step + 1;
            __threadfence();
        }
    }
    return;

abort:
    // a bounded wait gave up: record it, let this CTA's copies land (bounded)
    // so no TMA writes into released shared memory, and leave the counter
    if (tid == 0) {
        atomicOr(&P.ctl->status, 8);
        for (int s = 0; s < NSTAGE; ++s) {
            // copies still in flight on slot s complete phases uses[s] .. issued[s]-1
            for (uint32_t k = uses[s]; k < (uint32_t)issued[s]; ++k)
                for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
                    if (mbar_try_wait(&bars[s], k & 1u)) break;
        }
    }
    __syncthreads();
}

}  // namespace bt
