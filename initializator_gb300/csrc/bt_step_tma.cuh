// FP32 fast path of the fused step (K1, TMA form) for sm_103a.
//
// Same update and M(t) as step_kernel (bt_step.cuh), for steps without pulses
// and steps whose pulses are all fixed-angle (the RF instances apply the
// step's product rotation to each voxel's lab-frame value before the sums):
//   * a CTA owns a 128 x 8 column tile (64 x 16 for grids a 128-wide tile
//     would pad more: see Tile) and marches through a z-chunk (the first
//     P.zlong columns split into P.zsplit even chunks, the others into one
//     fewer; odd chunks march downwards, so the plane two neighbouring chunks
//     share is read by both at about the same moment and the second read hits
//     L2);
//   * each z-plane of the tile (the three field components with a one-voxel
//     x/y halo, upwind cell velocities, geometry code) is fetched by one thread with
//     cp.async.bulk.tensor into a 3-slot shared-memory ring, completion
//     tracked by one "full" mbarrier per slot (expect_tx), so two planes are
//     in flight while the CTA computes the current one; each warp releases a
//     slot through the slot's "empty" mbarrier (one arrival per warp) and only
//     the producing thread waits for it, so the warps of a CTA drift up to two
//     planes apart instead of meeting at a CTA barrier every plane;
//   * each thread computes 4 consecutive voxels along x (a warp holds one
//     row of a 128-wide tile or two rows of a 64-wide one): 128-bit shared
//     loads, 128-bit global stores; the voxel's own z-column (below / current
//     / above) rolls through registers;
//   * the stencil is evaluated as relaxation + sum over the six faces of
//     w_f * (M_f - M_0), w_f folding harmonic-mean diffusion and first-order
//     upwind advection; on a domain face the neighbour is the reference's
//     copy ghost (cpp:1664-1754), the voxel itself (rotated by the face phase
//     in the k frame), set once per plane in the few threads holding such a
//     face, so the face contributes nothing up to FP32 rounding and no
//     per-voxel weight zeroing is needed — FP32 only; the FP64 path keeps the
//     reference's exact operation order (and exact zero weights) in
//     step_kernel;
//   * the advection enters through one value per voxel and axis,
//     u = dt/(2 d) (v_lo + v_hi), zeroed where the face it draws from (v_hi
//     for u < 0, v_lo for u > 0) is closed; cell_velocity_kernel forms it once
//     per geometry upload with the same FP32 operations the per-face form
//     uses, so the weights are bit-identical to it and a plane's velocities
//     are one 3 x 128 x 8 box instead of three face boxes with halos;
//   * M(t) and the step counter: each CTA stores its FP64 partial (per-thread
//     Kahan, per-warp float-float, per-CTA FP64) into the partials buffer of
//     its input side; CTA 0 of the next fast step adds them in a fixed order
//     while its first planes load, and step_finish_kernel does so for the last
//     step of a run of fast steps. The first step of a run reads Ctl::step,
//     later ones the counter slot of their input side (Ctl::fstep), which the
//     previous step's CTA 0 wrote and which is read only after that grid has
//     completed; no CTA waits on a fence or an atomic ticket.
// Out-of-range TMA boxes (halo beyond the domain, plane -1 or nz) are
// zero-filled; a copy face replaces them by its ghost as described above, a
// zero face (bt_config.boundary) uses them as they are. Periodic faces (the
// BCK instances, KSPACE only) load the far edge: the wrapped plane by TMA in
// z, the far row / column by plain loads in the threads holding an edge in
// y / x, moved into the voxel's k frame by the step's wrap factor. The first
// step of a run from step 0 reads copy ghosts on every face, as the
// reference's initial ghost layer.
// Every mbarrier wait is bounded; a wait that gives up raises the CTA's
// failure flag, which ends the other warps' waits too; after the march the
// CTA then records status bit 8, drains its copies (bounded) and returns
// without storing its partial.
#pragma once
#include <cstdlib>

#include "bt_step.cuh"

namespace bt {

namespace tma {

constexpr int QX = 4;               // voxels per thread along x
constexpr int NT = 256;             // threads per CTA
constexpr int NWARP = NT / 32;      // warps per CTA (arrivals on an empty barrier)
constexpr int NSTAGE = 3;
constexpr int TAB_ROW = 12;         // floats per code-table row: 48 B, so 8 distinct rows hit 8 bank groups

// Tile geometry and shared-memory layout of the fast path for a tile TW
// voxels wide: 128 (one 32-lane warp per row, 8 rows) or 64 (16 lanes per
// row, two rows per warp, 16 rows) for narrow grids, where a 128-wide tile
// would leave many lanes idle. Every thread holds 4 voxels along x.
template <int TW_, bool PAL_ = false>
struct Tile {
    static_assert(TW_ == 128 || TW_ == 64, "tile width");
    static constexpr int TW = TW_;
    static constexpr int RPW = 128 / TW;          // rows per warp
    static constexpr int LW = 32 / RPW;           // lanes per row
    static constexpr int TH = NWARP * RPW;        // rows per tile
    static constexpr int SW = TW + 8;             // state tile width: x0-4 .. x0+TW+3
    static constexpr int SH = TH + 2;             // state tile height: y0-1 .. y0+TH
    static constexpr int OFF_STATE = 0;
    static constexpr int SZ_STATE = 3 * SH * SW * 4;
    static constexpr int OFF_U = (SZ_STATE + 127) / 128 * 128;
    static constexpr int SZ_U = 3 * TH * TW * 4;  // upwind cell velocities, 3 axes
    static constexpr int OFF_CODE = OFF_U + SZ_U;
    static constexpr int SZ_CODE = TH * TW;
    // per-voxel rate palette index (instances with per-voxel rates only)
    static constexpr int OFF_PAL = (OFF_CODE + SZ_CODE + 127) / 128 * 128;
    static constexpr int SZ_PAL = PAL_ ? TH * TW : 0;
    static constexpr int STAGE = (OFF_PAL + SZ_PAL + 127) / 128 * 128;
    static constexpr int OFF_AUX = NSTAGE * STAGE;  // tables, barriers, reduction
    // aux layout (bytes from OFF_AUX)
    static constexpr int AUX_TAB = 0;                     // 128 rows: 6 face weights, dt/T1, dt/T2, their sum, 3 unused
    static constexpr int AUX_EY = AUX_TAB + 128 * TAB_ROW * 4;  // exp(-i k_y y), TH float2
    static constexpr int AUX_BARS = AUX_EY + (8 * TH + 63) / 64 * 64;  // full[NSTAGE], empty[NSTAGE]
    static constexpr int AUX_FLAGS = AUX_BARS + 64;
    static constexpr int AUX_RED = AUX_FLAGS + 128;       // 8 warps x 3 doubles
    static constexpr int AUX_EX = AUX_RED + 256;          // exp(-i k_x x), TW float2
    static constexpr int AUX_EZ = AUX_EX + 8 * TW;        // exp(-i k_z z), up to ZCHUNK_MAX float2
    static constexpr int AUX_PAL = AUX_EZ + 8 * ZCHUNK_MAX;  // rate palette: 256 (dt/T1, dt/T2) float2
    static constexpr int SMEM = OFF_AUX + AUX_PAL + (PAL_ ? 8 * 256 : 0) + 128;  // + 128 for the base alignment
    static_assert(OFF_U % 128 == 0 && OFF_CODE % 128 == 0 && STAGE % 128 == 0, "TMA destinations 128-aligned");
    static_assert(TW + TH <= NT, "one phase-table entry per thread for x and y");
};
// the 128-wide tile keeps the layout the fast path was tuned with
static_assert(Tile<128>::OFF_U == 16384 && Tile<128>::STAGE == 29696 && Tile<128>::AUX_BARS == 6208, "layout");
// the drain after a give-up always waits this long (polls) for the copies in
// flight, so that no bulk copy lands in a CTA that has already exited
constexpr uint32_t WAIT_LIMIT = RING_WAIT_POLLS;

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sa(bar)) : "memory");
}
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
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(sa(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3, int c4) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
        "[%7];" ::"r"(sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(sa(bar))
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

// one thread per voxel (grid-stride): the fast path's gated cell velocities
// u[axis][z][y][pitch]; face arrays as StepParams describes them
static __global__ void cell_velocity_kernel(const StepParams<float> P, float* __restrict__ u, long long comp) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const float h2[3] = {0.5f * P.hx, 0.5f * P.hy, 0.5f * P.hz};
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q % nx);
        const long long r = q / nx;  // z * ny + y
        const int y = (int)(r % ny), z = (int)(r / ny);
        const float lo[3] = {P.vx[r * P.vxpitch + x], P.vy[((long long)z * (ny + 1) + y) * P.pitch + x],
                             P.vz[r * P.pitch + x]};
        const float hi[3] = {P.vx[r * P.vxpitch + x + 1], P.vy[((long long)z * (ny + 1) + y + 1) * P.pitch + x],
                             P.vz[(r + ny) * P.pitch + x]};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float v = h2[a] * (lo[a] + hi[a]);
            u[a * comp + r * P.pitch + x] = (v < 0.f ? hi[a] != 0.f : lo[a] != 0.f) ? v : 0.f;
        }
    }
}

template <int SCHEME, bool VEL, bool PREC, int TWV, bool BCK, int PH, bool PAL, bool RF>
__global__ void __launch_bounds__(tma::NT, 2)
    step_tma_kernel(const __grid_constant__ StepParams<float> P, const __grid_constant__ TmaMaps M, int first) {
    using namespace tma;
    // KSPACE: which axes carry a face phase (the schedule's wave vector has a
    // component along them at some step): every axis (PH_ALL), z alone (PH_Z:
    // gradients along z only, as every PGSE workload here), or none (PH_NONE:
    // no gradient); an axis without one uses real face weights, a unit
    // lab-frame phase and the voxel itself as its copy ghost, which is exact
    constexpr bool phx = SCHEME == SCHEME_KSPACE && PH == PH_ALL;
    constexpr bool phz = SCHEME == SCHEME_KSPACE && PH != PH_NONE;
    constexpr bool ph_axis[3] = {phx, phx, phz};
    using Tl = Tile<TWV, PAL>;
    constexpr int TW = Tl::TW, TH = Tl::TH, LW = Tl::LW, RPW = Tl::RPW, SW = Tl::SW, SH = Tl::SH;
    constexpr int OFF_STATE = Tl::OFF_STATE, OFF_U = Tl::OFF_U, OFF_CODE = Tl::OFF_CODE, STAGE = Tl::STAGE;
    constexpr int SZ_STATE = Tl::SZ_STATE, SZ_U = Tl::SZ_U, SZ_CODE = Tl::SZ_CODE, OFF_AUX = Tl::OFF_AUX;
    constexpr int AUX_TAB = Tl::AUX_TAB, AUX_EY = Tl::AUX_EY, AUX_BARS = Tl::AUX_BARS, AUX_FLAGS = Tl::AUX_FLAGS;
    constexpr int AUX_RED = Tl::AUX_RED, AUX_EX = Tl::AUX_EX, AUX_EZ = Tl::AUX_EZ, AUX_PAL = Tl::AUX_PAL;
    constexpr int OFF_PAL = Tl::OFF_PAL, SZ_PAL = Tl::SZ_PAL;
    // TMA destinations must sit on 128-byte boundaries: align the dynamic
    // shared-memory base explicitly (the launch reserves 128 spare bytes)
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((128u - (sa(smem_raw) & 127u)) & 127u);
    float4* s_tab = reinterpret_cast<float4*>(smem + OFF_AUX + AUX_TAB);
    float2* s_ey = reinterpret_cast<float2*>(smem + OFF_AUX + AUX_EY);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + OFF_AUX + AUX_BARS);
    uint64_t* empties = bars + NSTAGE;
    int* s_flags = reinterpret_cast<int*>(smem + OFF_AUX + AUX_FLAGS);
    double* red = reinterpret_cast<double*>(smem + OFF_AUX + AUX_RED);
    float2* s_ex = reinterpret_cast<float2*>(smem + OFF_AUX + AUX_EX);
    float2* s_ez = reinterpret_cast<float2*>(smem + OFF_AUX + AUX_EZ);
    float2* s_pal = reinterpret_cast<float2*>(smem + OFF_AUX + AUX_PAL);
    // RF: the step's pulse rotation, three rows (in the flag block's spare bytes)
    float4* s_rot = reinterpret_cast<float4*>(smem + OFF_AUX + AUX_FLAGS + 16);
    static_assert(AUX_FLAGS + 16 + 3 * 16 <= AUX_RED, "rotation rows fit the flag block");

    const int tid = threadIdx.x;
    const int lane = tid & 31, w = tid >> 5;
    // this thread's row of the tile and lane within that row
    const int row = w * RPW + lane / LW, xl = lane % LW;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    // blockIdx.x walks the z-chunks of one tile. Odd chunks march downwards,
    // so the plane two neighbouring chunks share is read by both at the same
    // moment (both at their start, or both at their end) and the second read
    // hits L2 instead of DRAM.
    // blockIdx.x = batch member + nbatch * z-chunk: the members of a q-sweep
    // run side by side, so the geometry and velocity tiles they share come
    // from L2 after the first member's DRAM read
    const unsigned nb = P.nbatch > 1 ? (unsigned)P.nbatch : 1u;
    const unsigned b = blockIdx.x % nb;
    const int zc = (int)(blockIdx.x / nb);
    const int x0 = blockIdx.y * TW, y0 = blockIdx.z * TH;
    // this tile column's chunks: P.zsplit for the first P.zlong tiles (x
    // fastest), one fewer for the rest, whose last grid index is then empty;
    // so any chunk count can fill whole waves. Even chunks within a column
    // (lengths differ by at most one plane).
    const int nch = P.zsplit - ((int)(blockIdx.y + gridDim.y * blockIdx.z) >= P.zlong ? 1 : 0);
    const int z0 = zc < nch ? (int)((long long)zc * nz / nch) : 0;
    const int z1 = zc < nch ? (int)((long long)(zc + 1) * nz / nch) : 0;
    const int d = (zc & 1) ? -1 : 1;
    const int xb = x0 + QX * xl;  // first of this thread's 4 voxels
    const int y = y0 + row;

    uint32_t txbytes = SZ_STATE + SZ_CODE + SZ_PAL;
    if constexpr (VEL) txbytes += SZ_U;
    auto issue = [&](int slot, int plane) {
        uint64_t* bar = &bars[slot];
        unsigned char* base = smem + slot * STAGE;
        mbar_expect_tx(bar, txbytes);
        tma_load_5d(base + OFF_STATE, &M.state, bar, x0 - 4, y0 - 1, plane, 0, (int)b);
        if constexpr (VEL) tma_load_4d(base + OFF_U, &M.ucell, bar, x0, y0, plane, 0);
        tma_load_3d(base + OFF_CODE, &M.code, bar, x0, y0, plane);
        if constexpr (PAL) tma_load_3d(base + OFF_PAL, &M.pal, bar, x0, y0, plane);
    };
    // ghost-layer kinds of this step (BCK instances; the first step of a run
    // from step 0 reads copies), set once the step index is known
    int kx = BC_COPY, ky = BC_COPY, kz = BC_COPY;
    // plane sequence: q = 0 is the ghost-side plane, then the chunk in marching
    // order; a periodic z face takes the far edge plane instead of plane -1 / nz
    auto plane_of = [&](int q) {
        int pl = d > 0 ? z0 - 1 + q : z1 - q;
        if constexpr (BCK) {
            if (kz == BC_PERIODIC) pl = pl < 0 ? nz - 1 : (pl >= nz ? 0 : pl);
        }
        return pl;
    };
    // a CTA without a chunk (the short columns' last grid index) issues no
    // copy, waits on nothing and contributes zero sums
    const bool empty = z1 <= z0;
    const int nplanes = empty ? 0 : z1 - z0 + 2;
    // plane q lands in slot q % NSTAGE as that slot's (q / NSTAGE)-th phase
    int n_issued = 0;  // planes issued so far (thread 0), always in plane order
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) {
            mbar_init(&bars[s], 1);
            mbar_init(&empties[s], NWARP);
        }
        fence_mbar_init();
        s_flags[0] = 0;
    }
    // per-CTA table indexed by the voxel code (bit 6 pore, bits 0-5 solid
    // faces): six face diffusion weights, dt/T1, dt/T2, the weights' sum; all
    // zero for solid.
    // It depends on the launch's parameters only, so with programmatic
    // dependent launch it is built while the previous step still runs.
    if (tid < 128) {
        const int f = tid & 63;
        const bool pore = tid & 64;
        const float dm = (pore && P.diffusion) ? 1.f : 0.f;
        const float kx = P.hxx * P.dpp, ky = P.hyy * P.dpp, kz = P.hzz * P.dpp;
        const float sx = P.hxx * P.dps, sy = P.hyy * P.dps, sz = P.hzz * P.dps;
        s_tab[3 * tid] = make_float4(dm * ((f & 1) ? sx : kx), dm * ((f & 2) ? sx : kx), dm * ((f & 4) ? sy : ky),
                                     dm * ((f & 8) ? sy : ky));
        s_tab[3 * tid + 1] = make_float4(dm * ((f & 16) ? sz : kz), dm * ((f & 32) ? sz : kz),
                                         pore ? P.dtt1[f] : 0.f, pore ? P.dtt2[f] : 0.f);
        // the six diffusion weights' sum, added in the order the voxel loop
        // used to add them
        const float4 a = s_tab[3 * tid], c = s_tab[3 * tid + 1];
        s_tab[3 * tid + 2] = make_float4(((a.x + a.y) + (a.z + a.w)) + (c.x + c.y), 0.f, 0.f, 0.f);
    }
    // the rate palette (per-voxel rates): one pair per thread
    if constexpr (PAL) s_pal[tid] = make_float2(P.pal[2 * tid], P.pal[2 * tid + 1]);
    static_assert(!PAL || NT == 256, "one palette entry per thread");
    // everything below reads what the previous step wrote (the field, the
    // step counter): wait until that grid has completed and its writes are
    // visible (returns at once when this launch has no programmatic
    // dependency)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // the step index: from Ctl::step for the first step of a run of fast
    // steps, else from this side's slot, which the previous step's CTA 0
    // wrote; CTA 0 writes the other side's slot for the next step (read only
    // after this grid has completed, so no CTA of this step sees it change)
    const bool cta0 = (blockIdx.x | blockIdx.y | blockIdx.z) == 0;
    const long long step = first ? __ldcg(&P.ctl->step) : __ldcg(&P.ctl->fstep[P.side]);
    if (cta0 && tid == 0) P.ctl->fstep[1 - P.side] = step + 1;
    const StepInfo* si = P.steps + (step < P.nsched ? step : P.nsched) * nb + b;
    if constexpr (BCK) {
        if (step > 0) {
            kx = P.bc[0];
            ky = P.bc[1];
            kz = P.bc[2];
        }
    }
    // a pulse step: every pulse fixed-angle, their product rotation
    if constexpr (RF) {
        if (tid < 3) s_rot[tid] = make_float4(si->rotf[3 * tid], si->rotf[3 * tid + 1], si->rotf[3 * tid + 2], 0.f);
    }
    if (tid == 0)
        for (int q = 0; q < NSTAGE && q < nplanes; ++q) {
            issue(q, plane_of(q));
            n_issued++;
        }
    // lab-frame phases (KSPACE), FP64-reduced arguments, each computed once
    // per CTA: the tile's 128 columns by threads 0..127, its 8 rows by threads
    // 128..135, the chunk's planes by the threads from 136 on (wrapping)
    if constexpr (phx) {
        if (tid < TW) lab_phase<float>(si->knext[0], x0 + tid, P.dxd, s_ex[tid].x, s_ex[tid].y);
        else if (tid < TW + TH) lab_phase<float>(si->knext[1], y0 + tid - TW, P.dyd, s_ey[tid - TW].x, s_ey[tid - TW].y);
    }
    if constexpr (phz) {
        for (int q = (tid + NT - (TW + TH)) % NT; q < z1 - z0; q += NT)
            lab_phase<float>(si->knext[2], z0 + q, P.dzd, s_ez[q].x, s_ez[q].y);
    }
    // CTA 0 adds the previous step's partials (complete: that grid has
    // finished) into its M(t) row while its own first planes are in flight
    const unsigned nb_per = (unsigned)P.zsplit * gridDim.y * gridDim.z;
    if (cta0 && !first) reduce_members<float>(P, P.partials_prev, step - 1, nb_per, red);
    __syncthreads();
    float exr[QX] = {1.f, 1.f, 1.f, 1.f}, exi[QX] = {0.f, 0.f, 0.f, 0.f};
    if constexpr (phx) {
#pragma unroll
        for (int i = 0; i < QX; ++i) {
            const float2 e = s_ex[QX * xl + i];
            exr[i] = e.x;
            exi[i] = e.y;
        }
    }

    // per-step uniforms
    float gdx = 0.f, gdy = 0.f, gdz = 0.f;
    if constexpr (PREC && SCHEME == SCHEME_REF) {
        gdx = (float)(si->grad[0] * P.dxd);
        gdy = (float)(si->grad[1] * P.dyd);
        gdz = (float)(si->grad[2] * P.dzd);
    }
    float ph[3][2] = {{1.f, 0.f}, {1.f, 0.f}, {1.f, 0.f}};  // exp(+i k d) per axis; the + face uses its conjugate
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (ph_axis[a]) {
            ph[a][0] = si->phasef[a][0];
            ph[a][1] = si->phasef[a][1];
        }
    // summation mask of this thread's 4 voxels (trimming box, inside the grid)
    uint32_t xmask = 0;
#pragma unroll
    for (int i = 0; i < QX; ++i)
        if (xb + i < nx && xb + i >= P.box[0] && xb + i < P.box[1]) xmask |= 1u << i;
    const bool row_sum = y < ny && y >= P.box[2] && y < P.box[3];
    const bool row_ok = y < ny;
    // a warp whose rows all lie beyond the grid (the last tile row of a grid
    // whose height is not a multiple of the tile's) skips the arithmetic and
    // only keeps the ring going: its voxels are stored nowhere and add nothing
    const bool warp_rows = __any_sync(0xffffffffu, row_ok);
    // threads holding a voxel on a domain face in x (lane 0 of the first
    // tile, the thread holding x = nx - 1); rows on a face in y are warp-uniform
    const bool x_lo = xb == 0;
    const bool x_hi = xb <= nx - 1 && nx - 1 < xb + QX;

    Acc<float> acc[3];
    float prv[3][QX], cur[3][QX], nxt[3][QX];

    auto own = [&](int slot, float (&dst)[3][QX]) {
        const float* st = reinterpret_cast<const float*>(smem + slot * STAGE + OFF_STATE);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float4 v = *reinterpret_cast<const float4*>(st + (c * SH + row + 1) * SW + 4 + QX * xl);
            dst[c][0] = v.x; dst[c][1] = v.y; dst[c][2] = v.z; dst[c][3] = v.w;
        }
    };
    // s_flags[0] is the CTA's failure flag (volatile: polled inside waits)
    volatile int* vflag = s_flags;
    // Plane q of the sequence uses slot q % NSTAGE for the (q / NSTAGE)-th
    // time, so its full barrier completes phase (q / NSTAGE) & 1; the loop
    // carries slot and parity instead of dividing.
    // warp-uniform bounded wait for the copy into `slot` at phase parity
    // `par`; false when it gave up or another thread of the CTA raised the
    // failure flag
    const uint32_t polls = P.wait_polls;
    auto wait_full = [&](int slot, uint32_t par) -> bool {
        for (uint32_t i = 0; i < polls; ++i) {
            if (__all_sync(0xffffffffu, mbar_try_wait(&bars[slot], par))) return true;
            if (__any_sync(0xffffffffu, vflag[0] != 0)) return false;
        }
        if (lane == 0) vflag[0] = 1;
        return false;
    };
    // a warp is done with a slot
    auto release = [&](int slot) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empties[slot]);
    };
    // producer (thread 0): plane p into `slot` (= p % NSTAGE) once every warp
    // has released plane p - NSTAGE from it, whose phase parity is `par`
    // (bounded; raises the flag on timeout)
    auto refill = [&](int p, int slot, uint32_t par) {
        for (uint32_t i = 0; i < polls; ++i) {
            if (mbar_try_wait(&empties[slot], par)) {
                fence_proxy_async();
                issue(slot, plane_of(p));
                n_issued++;
                return;
            }
            if (vflag[0]) return;
        }
        vflag[0] = 1;
    };

    // prologue: the ghost-side plane (q = 0) and the first plane (q = 1)
    bool live = !empty;
    if (live) {
        live = wait_full(0, 0u);
        if (live) {
            own(0, prv);
            live = wait_full(1, 0u);
        }
        if (live) {
            own(1, cur);
            release(0);
            if (tid == 0 && nplanes > NSTAGE) refill(NSTAGE, 0, 0u);
        }
    }

    // the value a domain face's ghost must hold for the face to contribute
    // nothing (the reference's copy ghosts, cpp:1664-1754): the voxel itself,
    // in the k frame rotated so that the stencil's face phase (exp(+i th) on
    // the lower face, its conjugate on the upper) brings it back to the voxel
    auto ghost = [&](float& gr, float& gi, float& gz, float mr, float mi, float mz, int a, bool upper) {
        if (a == 2 ? phz : phx) {
            // selected, not indexed: a runtime index would put ph in local memory
            const float pc = a == 0 ? ph[0][0] : (a == 1 ? ph[1][0] : ph[2][0]);
            const float ps = a == 0 ? ph[0][1] : (a == 1 ? ph[1][1] : ph[2][1]);
            const float c = pc, s = upper ? -ps : ps;
            gr = c * mr + s * mi;
            gi = c * mi - s * mr;
        } else {
            gr = mr;
            gi = mi;
        }
        gz = mz;
    };
    auto ghost_plane = [&](float (&g)[3][QX], int a, bool upper) {
#pragma unroll
        for (int i = 0; i < QX; ++i) ghost(g[0][i], g[1][i], g[2][i], cur[0][i], cur[1][i], cur[2][i], a, upper);
    };
    // a periodic face's ghost: the far edge cell (mr, mi, mz) moved across the
    // period into the k frame (exp(-i k_a L_a) below, its conjugate above)
    auto wrap = [&](float& gr, float& gi, float& gz, float mr, float mi, float mz, int a, bool upper) {
        if constexpr (SCHEME == SCHEME_KSPACE) {
            const float c = si->wrapf[a][0], s_ = upper ? -si->wrapf[a][1] : si->wrapf[a][1];
            gr = c * mr - s_ * mi;
            gi = c * mi + s_ * mr;
        } else {
            gr = mr;
            gi = mi;
        }
        gz = mz;
    };
    // input field of this member (periodic faces read the far edge directly)
    const float* fin[3] = {P.in[0] + (long long)b * P.bstride, P.in[1] + (long long)b * P.bstride,
                           P.in[2] + (long long)b * P.bstride};

    // output offset of this thread's row in plane 0
    const long long obase = (long long)b * P.bstride + (long long)y * P.pitch + xb;
    int sc = 1;         // slot of plane q
    uint32_t pc = 0u;   // its phase parity
    // M(t) summation mask: fixed for the whole chunk unless the trimming box
    // cuts it in z (never for the default box)
    const uint32_t smask_row = row_sum ? xmask : 0u;
    const bool z_trim = !(z0 >= P.box[4] && z1 <= P.box[5]);
    int z = plane_of(1);
    for (int q = 1; live && q + 1 < nplanes; ++q, z += d) {
        const int sn = sc == NSTAGE - 1 ? 0 : sc + 1;   // slot of plane q + 1
        const uint32_t pn = sc == NSTAGE - 1 ? pc ^ 1u : pc;
        if (!wait_full(sn, pn)) break;
        own(sn, nxt);
        // one instance of the plane body per marching direction, so that
        // below / above bind to fixed registers
        auto body = [&](const float(&bel)[3][QX], const float(&abv)[3][QX]) {
        const unsigned char* base = smem + sc * STAGE;
        const float* st = reinterpret_cast<const float*>(base + OFF_STATE);
        float xm[3][QX], xp[3][QX], ym[3][QX], yp[3][QX];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* rp = st + (c * SH + row + 1) * SW + 4 + QX * xl;
            const float4 a = *reinterpret_cast<const float4*>(rp - SW);
            const float4 b = *reinterpret_cast<const float4*>(rp + SW);
            ym[c][0] = a.x; ym[c][1] = a.y; ym[c][2] = a.z; ym[c][3] = a.w;
            yp[c][0] = b.x; yp[c][1] = b.y; yp[c][2] = b.z; yp[c][3] = b.w;
            // x halo from the neighbouring lanes; only the tile edges read shared
            // memory (a stride-16-byte scalar load by every lane conflicts 4 ways)
            float l = __shfl_up_sync(0xffffffffu, cur[c][QX - 1], 1, LW);
            float r = __shfl_down_sync(0xffffffffu, cur[c][0], 1, LW);
            if (xl == 0) l = rp[-1];
            if (xl == LW - 1) r = rp[QX];
            xm[c][0] = l;
            xp[c][QX - 1] = r;
#pragma unroll
            for (int i = 1; i < QX; ++i) xm[c][i] = cur[c][i - 1];
#pragma unroll
            for (int i = 0; i < QX - 1; ++i) xp[c][i] = cur[c][i + 1];
        }
        // voxels on a domain face in x or y: the halo value beyond the face
        // (zero-filled by the copy) becomes the face's ghost, so no weight
        // needs zeroing per voxel
        // (a zero face keeps the zero-filled halo)
        const long long zoff = (long long)z * P.plane;
        if (x_lo) {
            if (kx == BC_COPY) ghost(xm[0][0], xm[1][0], xm[2][0], cur[0][0], cur[1][0], cur[2][0], 0, false);
            if constexpr (BCK) {
                if (kx == BC_PERIODIC) {
                    const long long o = zoff + (long long)y * P.pitch + (nx - 1);
                    wrap(xm[0][0], xm[1][0], xm[2][0], fin[0][o], fin[1][o], fin[2][o], 0, false);
                }
            }
        }
        if (x_hi) {
#pragma unroll
            for (int i = 0; i < QX; ++i)
                if (xb + i == nx - 1) {
                    if (kx == BC_COPY) ghost(xp[0][i], xp[1][i], xp[2][i], cur[0][i], cur[1][i], cur[2][i], 0, true);
                    if constexpr (BCK) {
                        if (kx == BC_PERIODIC) {
                            const long long o = zoff + (long long)y * P.pitch;
                            wrap(xp[0][i], xp[1][i], xp[2][i], fin[0][o], fin[1][o], fin[2][o], 0, true);
                        }
                    }
                }
        }
        if (y == 0) {
            if (ky == BC_COPY) {
#pragma unroll
                for (int i = 0; i < QX; ++i)
                    ghost(ym[0][i], ym[1][i], ym[2][i], cur[0][i], cur[1][i], cur[2][i], 1, false);
            }
            if constexpr (BCK) {
                if (ky == BC_PERIODIC) {
                    const long long o = zoff + (long long)(ny - 1) * P.pitch + xb;
                    float f[3][QX];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float4 v = *reinterpret_cast<const float4*>(fin[c] + o);
                        f[c][0] = v.x; f[c][1] = v.y; f[c][2] = v.z; f[c][3] = v.w;
                    }
#pragma unroll
                    for (int i = 0; i < QX; ++i) wrap(ym[0][i], ym[1][i], ym[2][i], f[0][i], f[1][i], f[2][i], 1, false);
                }
            }
        }
        if (y == ny - 1) {
            if (ky == BC_COPY) {
#pragma unroll
                for (int i = 0; i < QX; ++i)
                    ghost(yp[0][i], yp[1][i], yp[2][i], cur[0][i], cur[1][i], cur[2][i], 1, true);
            }
            if constexpr (BCK) {
                if (ky == BC_PERIODIC) {
                    const long long o = zoff + xb;
                    float f[3][QX];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float4 v = *reinterpret_cast<const float4*>(fin[c] + o);
                        f[c][0] = v.x; f[c][1] = v.y; f[c][2] = v.z; f[c][3] = v.w;
                    }
#pragma unroll
                    for (int i = 0; i < QX; ++i) wrap(yp[0][i], yp[1][i], yp[2][i], f[0][i], f[1][i], f[2][i], 1, true);
                }
            }
        }
        const uint32_t code4 = *reinterpret_cast<const uint32_t*>(base + OFF_CODE + row * TW + QX * xl);
        uint32_t pal4 = 0;
        if constexpr (PAL) pal4 = *reinterpret_cast<const uint32_t*>(base + OFF_PAL + row * TW + QX * xl);
        float ux[QX] = {0.f, 0.f, 0.f, 0.f}, uy[QX] = {0.f, 0.f, 0.f, 0.f}, uz[QX] = {0.f, 0.f, 0.f, 0.f};
        if constexpr (VEL) {
            const float* ur = reinterpret_cast<const float*>(base + OFF_U) + row * TW + QX * xl;
            const float4 a = *reinterpret_cast<const float4*>(ur);
            const float4 b = *reinterpret_cast<const float4*>(ur + TH * TW);
            const float4 c = *reinterpret_cast<const float4*>(ur + 2 * TH * TW);
            ux[0] = a.x; ux[1] = a.y; ux[2] = a.z; ux[3] = a.w;
            uy[0] = b.x; uy[1] = b.y; uy[2] = b.z; uy[3] = b.w;
            uz[0] = c.x; uz[1] = c.y; uz[2] = c.z; uz[3] = c.w;
        }
        uint32_t smask = smask_row;
        if (z_trim && (z < P.box[4] || z >= P.box[5])) smask = 0u;
        float o[3][QX];
        float sx_r = 0.f, sx_i = 0.f, sz_ = 0.f;  // this plane's sums over the 4 voxels
        // RF, KSPACE: exp(-i (k_y y + k_z z)) of this row and plane
        float rer = 1.f, rei = 0.f;
        if constexpr (RF && SCHEME == SCHEME_KSPACE) {
            if constexpr (phx) {
                const float2 ey = s_ey[row], ez = s_ez[z - z0];
                rer = ey.x * ez.x - ey.y * ez.y;
                rei = ey.x * ez.y + ey.y * ez.x;
            } else if constexpr (phz) {
                const float2 ez = s_ez[z - z0];
                rer = ez.x;
                rei = ez.y;
            }
        }
#pragma unroll
        for (int i = 0; i < QX; ++i) {
            const uint32_t cd = (code4 >> (8 * i)) & 127u;
            const float4 ta = s_tab[3 * cd], tb = s_tab[3 * cd + 1];
            float wxm = ta.x, wxp = ta.y, wym = ta.z, wyp = ta.w, wzm = tb.x, wzp = tb.y;
            float dtt1 = tb.z, dtt2 = tb.w;
            if constexpr (PAL) {
                // per-voxel rates: the voxel's palette entry
                const float2 r = s_pal[(pal4 >> (8 * i)) & 255u];
                dtt1 = r.x;
                dtt2 = r.y;
            }
            if constexpr (VEL) {
                // upwind: +face -min(u,0), -face +max(u,0), u the gated cell
                // average (zero where the face it draws from is closed)
                wxp -= fminf(ux[i], 0.f);
                wxm += fmaxf(ux[i], 0.f);
                wyp -= fminf(uy[i], 0.f);
                wym += fmaxf(uy[i], 0.f);
                wzp -= fminf(uz[i], 0.f);
                wzm += fmaxf(uz[i], 0.f);
            }
            // the sum of the six face weights: the diffusion part from the
            // table; upwind adds max(u, 0) - min(u, 0) = |u| per axis
            float wsum = reinterpret_cast<const float*>(s_tab + 3 * cd + 2)[0];
            if constexpr (VEL) wsum = ((wsum + fabsf(ux[i])) + fabsf(uy[i])) + fabsf(uz[i]);
            const float px0 = cur[0][i], py0 = cur[1][i], pz0 = cur[2][i];
            float ax, ay, az;
            if constexpr (SCHEME == SCHEME_REF) {
                const float div = P.an[0] * px0 + P.an[1] * py0 + P.an[2] * pz0;
                const float divx = P.an[0] * div, divy = P.an[1] * div, divz = P.an[2] * div;
                ax = px0 + dtt1 * (P.peqn[0] - divx) + dtt2 * (divx - px0);
                ay = py0 + dtt1 * (P.peqn[1] - divy) + dtt2 * (divy - py0);
                az = pz0 + dtt1 * (P.peqn[2] - divz) + dtt2 * (divz - pz0);
                if constexpr (PREC) {
                    const float bbxb = P.b * (gdx * ((float)(xb + i) + 0.5f));
                    const float bbyb = P.b * (gdy * ((float)y + 0.5f));
                    const float bbzb = P.b * (gdz * ((float)z + 0.5f));
                    ax += bbzb * py0 - bbyb * pz0;
                    ay += bbxb * pz0 - bbzb * px0;
                    az += bbyb * px0 - bbxb * py0;
                }
                ax += wxm * xm[0][i] + wxp * xp[0][i] + wym * ym[0][i] + wyp * yp[0][i] + wzm * bel[0][i] +
                      wzp * abv[0][i] - wsum * px0;
                ay += wxm * xm[1][i] + wxp * xp[1][i] + wym * ym[1][i] + wyp * yp[1][i] + wzm * bel[1][i] +
                      wzp * abv[1][i] - wsum * py0;
            } else {
                ax = px0 - dtt2 * px0;
                ay = py0 - dtt2 * py0;
                az = pz0 + dtt1 * (P.peqn[2] - pz0);
                // per axis: w- e^{+i th} m- + w+ e^{-i th} m+
                //   = cos th (p + q) + i sin th (p - q),  p = w- m-, q = w+ m+
                auto axis = [&](float wm, float wp, float mr, float mi, float pr_, float pi_, float c, float s_,
                                float& accr, float& acci) {
                    const float pr = wm * mr, pi = wm * mi, qr = wp * pr_, qi = wp * pi_;
                    const float ar = pr + qr, ai = pi + qi, br = pr - qr, bi = pi - qi;
                    accr += c * ar - s_ * bi;
                    acci += c * ai + s_ * br;
                };
                // an axis without a phase: real weights on both parts
                auto axis_real = [&](float wm, float wp, float mr, float mi, float pr_, float pi_, float& accr,
                                     float& acci) {
                    accr += wm * mr + wp * pr_;
                    acci += wm * mi + wp * pi_;
                };
                float tr = -wsum * px0, ti = -wsum * py0;
                if constexpr (phx) {
                    axis(wxm, wxp, xm[0][i], xm[1][i], xp[0][i], xp[1][i], ph[0][0], ph[0][1], tr, ti);
                    axis(wym, wyp, ym[0][i], ym[1][i], yp[0][i], yp[1][i], ph[1][0], ph[1][1], tr, ti);
                } else {
                    axis_real(wxm, wxp, xm[0][i], xm[1][i], xp[0][i], xp[1][i], tr, ti);
                    axis_real(wym, wyp, ym[0][i], ym[1][i], yp[0][i], yp[1][i], tr, ti);
                }
                if constexpr (phz) axis(wzm, wzp, bel[0][i], bel[1][i], abv[0][i], abv[1][i], ph[2][0], ph[2][1], tr, ti);
                else axis_real(wzm, wzp, bel[0][i], bel[1][i], abv[0][i], abv[1][i], tr, ti);
                ax += tr;
                ay += ti;
            }
            az += wxm * xm[2][i] + wxp * xp[2][i] + wym * ym[2][i] + wyp * yp[2][i] + wzm * bel[2][i] +
                  wzp * abv[2][i] - wsum * pz0;
            const bool pore = cd & CODE_PORE;
            o[0][i] = pore ? ax : 0.f;
            o[1][i] = pore ? ay : 0.f;
            o[2][i] = pore ? az : 0.f;
            if constexpr (RF) {
                // the step's pulses act on the lab-frame value m_lab = e m,
                // e = exp(-i k.r) this voxel's frame factor (1 for the
                // reference scheme), and the result goes back: m = conj(e) m_lab
                float er = rer, ei = rei, lr = o[0][i], li = o[1][i];
                if constexpr (SCHEME == SCHEME_KSPACE) {
                    if constexpr (phx) {
                        er = exr[i] * rer - exi[i] * rei;
                        ei = exr[i] * rei + exi[i] * rer;
                    }
                    lr = er * o[0][i] - ei * o[1][i];
                    li = er * o[1][i] + ei * o[0][i];
                }
                const float lz = o[2][i];
                const float4 r0 = s_rot[0], r1 = s_rot[1], r2 = s_rot[2];
                const float nr = r0.x * lr + r0.y * li + r0.z * lz;
                const float ni = r1.x * lr + r1.y * li + r1.z * lz;
                o[2][i] = r2.x * lr + r2.y * li + r2.z * lz;
                if constexpr (SCHEME == SCHEME_KSPACE) {
                    o[0][i] = er * nr + ei * ni;
                    o[1][i] = er * ni - ei * nr;
                } else {
                    o[0][i] = nr;
                    o[1][i] = ni;
                }
            }
            const bool take = (smask >> i) & 1u;
            const float mr = take ? o[0][i] : 0.f, mi = take ? o[1][i] : 0.f;
            if constexpr (phx) {
                sx_r += exr[i] * mr - exi[i] * mi;
                sx_i += exr[i] * mi + exi[i] * mr;
            } else {
                sx_r += mr;
                sx_i += mi;
            }
            sz_ += take ? o[2][i] : 0.f;
        }
        if constexpr (phx) {
            // lab frame: multiply the row sum by exp(-i k_y y) exp(-i k_z z)
            const float2 ey = s_ey[row], ez = s_ez[z - z0];
            const float er = ey.x * ez.x - ey.y * ez.y, ei = ey.x * ez.y + ey.y * ez.x;
            acc[0].add(er * sx_r - ei * sx_i);
            acc[1].add(er * sx_i + ei * sx_r);
        } else if constexpr (phz) {
            const float2 ez = s_ez[z - z0];
            acc[0].add(ez.x * sx_r - ez.y * sx_i);
            acc[1].add(ez.x * sx_i + ez.y * sx_r);
        } else {
            acc[0].add(sx_r);
            acc[1].add(sx_i);
        }
        acc[2].add(sz_);
        if (row_ok && xb < nx) {
            const long long off = obase + (long long)z * P.plane;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                *reinterpret_cast<float4*>(P.out[c] + off) = make_float4(o[c][0], o[c][1], o[c][2], o[c][3]);
        }
        };
        // planes on a domain face in z: the ghost plane beyond it (zero-filled
        // by the copy, used by nothing else) becomes the face's ghost; on a
        // periodic face it is the far edge plane, moved into the k frame
        if (z == 0) {
            if (kz == BC_COPY) ghost_plane(d > 0 ? prv : nxt, 2, false);
            if constexpr (BCK) {
                if (kz == BC_PERIODIC) {
                    float (&g)[3][QX] = d > 0 ? prv : nxt;
#pragma unroll
                    for (int i = 0; i < QX; ++i) wrap(g[0][i], g[1][i], g[2][i], g[0][i], g[1][i], g[2][i], 2, false);
                }
            }
        }
        if (z == nz - 1) {
            if (kz == BC_COPY) ghost_plane(d > 0 ? nxt : prv, 2, true);
            if constexpr (BCK) {
                if (kz == BC_PERIODIC) {
                    float (&g)[3][QX] = d > 0 ? nxt : prv;
#pragma unroll
                    for (int i = 0; i < QX; ++i) wrap(g[0][i], g[1][i], g[2][i], g[0][i], g[1][i], g[2][i], 2, true);
                }
            }
        }
        if (warp_rows) {
            if (d > 0) body(prv, nxt);
            else body(nxt, prv);
        }
        release(sc);
        if (tid == 0 && q + NSTAGE < nplanes) refill(q + NSTAGE, sc, pc);
        sc = sn;
        pc = pn;
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int i = 0; i < QX; ++i) {
                prv[c][i] = cur[c][i];
                cur[c][i] = nxt[c][i];
            }
    }

    // this CTA has read all its input: the next step's grid may start its
    // CTAs (they build their tables, then wait for this grid to complete)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // the flag is only written inside the march: after this barrier every
    // thread sees its final value, so the branch below is CTA-uniform
    __syncthreads();
    if (vflag[0]) goto abort;

    // ---- deterministic M(t) reduction (as step_kernel) ----
    {
        const unsigned local = (unsigned)zc + (unsigned)P.zsplit * (blockIdx.y + gridDim.y * blockIdx.z);
        cta_partial_acc(P, b, local, nb_per, acc, red);
    }
    return;

abort:
    // a bounded wait gave up: record it, let this CTA's copies land (bounded)
    // so no TMA writes into released shared memory, and leave the counter
    if (tid == 0) {
        atomicOr(&P.ctl->status, 8);
        // the last NSTAGE planes issued may still be in flight: wait (bounded)
        // for the latest phase of each slot
        for (int q = max(0, n_issued - NSTAGE); q < n_issued; ++q)
            for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
                if (mbar_try_wait(&bars[q % NSTAGE], (uint32_t)(q / NSTAGE) & 1u)) break;
    }
    __syncthreads();
}

// programmatic dependent launch: a kernel overlaps its step-independent
// prologue with the previous launch's tail (BT_NO_PDL turns it off)
static inline cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, int smem, cudaStream_t s,
                                            cudaLaunchAttribute* attr) {
    static const bool pdl = std::getenv("BT_NO_PDL") == nullptr;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cfg;
}

template <int SCHEME, bool VEL, bool PREC, int TWV, bool BCK = false, int PH = PH_ALL, bool PAL = false,
          bool RF = false>
static cudaError_t launch_tma_t(const StepParams<float>& p, const TmaMaps& m, dim3 grid, bool first, cudaStream_t s) {
    constexpr int smem = tma::Tile<TWV, PAL>::SMEM;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(step_tma_kernel<SCHEME, VEL, PREC, TWV, BCK, PH, PAL, RF>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = pdl_config(grid, dim3(tma::NT), smem, s, attr);
    return cudaLaunchKernelEx(&cfg, step_tma_kernel<SCHEME, VEL, PREC, TWV, BCK, PH, PAL, RF>, p, m, first ? 1 : 0);
}

// per-voxel rates (the rate palette): the reference scheme, and KSPACE with
// copy faces
template <int TWV>
static cudaError_t launch_step_tma_pal(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec,
                                       dim3 grid, bool first, cudaStream_t s) {
    if (scheme == SCHEME_REF) {
        if (vel && prec) return launch_tma_t<SCHEME_REF, true, true, TWV, false, PH_ALL, true>(p, m, grid, first, s);
        if (vel) return launch_tma_t<SCHEME_REF, true, false, TWV, false, PH_ALL, true>(p, m, grid, first, s);
        if (prec) return launch_tma_t<SCHEME_REF, false, true, TWV, false, PH_ALL, true>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_REF, false, false, TWV, false, PH_ALL, true>(p, m, grid, first, s);
    }
    if (p.phase_axes == PH_Z) {
        if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_Z, true>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_Z, true>(p, m, grid, first, s);
    }
    if (p.phase_axes == PH_NONE) {
        if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_NONE, true>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_NONE, true>(p, m, grid, first, s);
    }
    if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_ALL, true>(p, m, grid, first, s);
    return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_ALL, true>(p, m, grid, first, s);
}

// pulse steps of the fast path (every pulse of the step fixed-angle): KSPACE
// with copy faces takes the instance of its phase axes when they are z or
// none (PGSE and multi-echo schedules), else the general one (any phase axes,
// any faces)
template <int TWV>
static cudaError_t launch_step_tma_rfw(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec,
                                       dim3 grid, bool first, cudaStream_t s) {
    if (scheme == SCHEME_REF) {
        if (vel && prec) return launch_tma_t<SCHEME_REF, true, true, TWV, false, PH_ALL, false, true>(p, m, grid, first, s);
        if (vel) return launch_tma_t<SCHEME_REF, true, false, TWV, false, PH_ALL, false, true>(p, m, grid, first, s);
        if (prec) return launch_tma_t<SCHEME_REF, false, true, TWV, false, PH_ALL, false, true>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_REF, false, false, TWV, false, PH_ALL, false, true>(p, m, grid, first, s);
    }
    if (p.bc[0] == BC_COPY && p.bc[1] == BC_COPY && p.bc[2] == BC_COPY) {
        if (p.phase_axes == PH_Z) {
            if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_Z, false, true>(p, m, grid, first, s);
            return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_Z, false, true>(p, m, grid, first, s);
        }
        if (p.phase_axes == PH_NONE) {
            if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_NONE, false, true>(p, m, grid, first, s);
            return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_NONE, false, true>(p, m, grid, first, s);
        }
    }
    if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, true, PH_ALL, false, true>(p, m, grid, first, s);
    return launch_tma_t<SCHEME_KSPACE, false, false, TWV, true, PH_ALL, false, true>(p, m, grid, first, s);
}

// the fast path's kernels of one tile width
template <int TWV>
static cudaError_t launch_step_tma_w(const StepParams<float>& p, const TmaMaps& m, int scheme, int vel, int prec,
                                     dim3 grid, bool first, cudaStream_t s) {
    if (scheme == SCHEME_REF) {
        if (vel && prec) return launch_tma_t<SCHEME_REF, true, true, TWV>(p, m, grid, first, s);
        if (vel) return launch_tma_t<SCHEME_REF, true, false, TWV>(p, m, grid, first, s);
        if (prec) return launch_tma_t<SCHEME_REF, false, true, TWV>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_REF, false, false, TWV>(p, m, grid, first, s);
    }
    // KSPACE with a non-copy face: the instance that reads the far edge
    if (p.bc[0] != BC_COPY || p.bc[1] != BC_COPY || p.bc[2] != BC_COPY) {
        if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, true>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_KSPACE, false, false, TWV, true>(p, m, grid, first, s);
    }
    // the phase axes of the schedule (bt_api.cu sets p.phase_axes)
    if (p.phase_axes == PH_Z) {
        if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_Z>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_Z>(p, m, grid, first, s);
    }
    if (p.phase_axes == PH_NONE) {
        if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV, false, PH_NONE>(p, m, grid, first, s);
        return launch_tma_t<SCHEME_KSPACE, false, false, TWV, false, PH_NONE>(p, m, grid, first, s);
    }
    if (vel) return launch_tma_t<SCHEME_KSPACE, true, false, TWV>(p, m, grid, first, s);
    return launch_tma_t<SCHEME_KSPACE, false, false, TWV>(p, m, grid, first, s);
}

}  // namespace bt
