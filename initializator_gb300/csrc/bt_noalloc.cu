// bt_step_noalloc: one step of the reference update that performs no device
// allocation at all.
//
// Who needs this: callers that may not call cudaMalloc — code that runs while
// a CUDA stream is being captured into a graph (allocation is not a stream
// operation and breaks the capture), host applications whose framework has
// already reserved (almost) all device memory for its own pool, and
// plugin hosts that forbid libraries from allocating behind their back. Such a
// caller owns every input and output buffer and passes them in; this entry
// point needs no handle and allocates nothing.
//
// The step itself is the library's generic fused kernel (step_kernel in
// bt_step.cuh, the same code the handle-based API runs for FP64 and for steps
// that carry pulses). Its scratch — the run-control block (step counter, CTA
// ticket), the per-step schedule record, the per-CTA partial sums of M(t) and
// the per-voxel geometry code derived from the mask — lives in the file-scope
// array below instead of in memory allocated by bt_create. Every GPU that
// loads the library holds that array until the process exits.
//
// Sharing: all calls on a device use the same array, and the array keeps the
// previous call's contents. Each call clears what must start at zero (the
// run-control block) and rebuilds the rest before its step kernel reads it,
// so sequential calls are independent. Calls whose kernels overlap on the GPU
// (different streams, or different host threads, without ordering between
// them) race on the array and give wrong results: order them on one stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "../../include/bt.h"
#include "bt_internal.h"

namespace {

constexpr size_t OFF_CTL = 0;                                     // bt::Ctl
constexpr size_t OFF_STEP = 256;                                  // one bt::StepInfo
constexpr size_t OFF_PULSE = 768;                                 // one bt::DevPulse
constexpr size_t OFF_PARTIALS = 1024;                             // 3 doubles per CTA
constexpr size_t OFF_CODE = OFF_PARTIALS + 3 * sizeof(double) * BT_NOALLOC_MAX_BLOCKS;
constexpr size_t SCRATCH_BYTES = OFF_CODE + BT_NOALLOC_MAX_VOXELS;
static_assert(sizeof(bt::Ctl) <= OFF_STEP - OFF_CTL, "layout");
static_assert(sizeof(bt::StepInfo) <= OFF_PULSE - OFF_STEP, "layout");
static_assert(sizeof(bt::DevPulse) <= OFF_PARTIALS - OFF_PULSE, "layout");

// The scratch of every allocation-free call on this device (about 2.4 MB).
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
// per device: the device address of the array and the id of the context it
// was looked up in (a cudaDeviceReset ends that context; the module is loaded
// again in the next one and the array may move)
unsigned char* g_scratch_addr[MAX_DEVICES] = {};
unsigned long long g_scratch_ctx[MAX_DEVICES] = {};

// unique id of the calling thread's current context (0 when there is none or
// the driver cannot say)
unsigned long long current_context_id() {
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static bool looked = false;
    if (!looked) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
        looked = true;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Set-up, once per device and context, with that device current: the
// host-side name of a __device__ array is only a stand-in; the address a
// kernel may use comes from cudaGetSymbolAddress (which also creates the
// device's context on a first call).
// The look-up is not a stream operation; a call whose look-up would fall
// inside a stream capture is refused (cudaErrorStreamCaptureUnsupported), so
// the rule that the first call on a device precedes any capture is enforced.
cudaError_t scratch_for_current_device(cudaStream_t stream, unsigned char** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
            return cudaErrorStreamCaptureUnsupported;
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
        g_scratch_ctx[dev] = current_context_id();
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

// the geometry code of the kernels (bit f: in-domain solid face neighbour
// -x,+x,-y,+y,-z,+z; bit 6: pore) from a dense mask, into the scratch array
__global__ void noalloc_code_kernel(const uint8_t* mask, uint8_t* code, int nx, int ny, int nz) {
    const long long n = (long long)nx * ny * nz;
    const long long plane = (long long)nx * ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q % nx), y = (int)((q / nx) % ny), z = (int)(q / plane);
        uint8_t c = 0;
        if (mask[q]) {
            c = bt::CODE_PORE;
            if (x > 0 && !mask[q - 1]) c |= 1;
            if (x < nx - 1 && !mask[q + 1]) c |= 2;
            if (y > 0 && !mask[q - nx]) c |= 4;
            if (y < ny - 1 && !mask[q + nx]) c |= 8;
            if (z > 0 && !mask[q - plane]) c |= 16;
            if (z < nz - 1 && !mask[q + plane]) c |= 32;
        }
        code[q] = c;
    }
}

// the schedule record of the single step: static gradient, no pulses
__global__ void noalloc_step_record_kernel(bt::StepInfo* si, bt::DevPulse* pu, double gx, double gy, double gz) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    si->grad[0] = gx;
    si->grad[1] = gy;
    si->grad[2] = gz;
    for (int a = 0; a < 3; ++a) si->knext[a] = 0.0;
    for (int f = 0; f < 6; ++f) {
        si->phase[f][0] = 1.0;
        si->phase[f][1] = 0.0;
    }
    si->pulse_first = 0;
    si->pulse_count = 0;
    pu->flag = 0;
}

template <typename T>
void fill(const bt_config& c, bt::StepParams<T>& P, const void* const in[3], void* const out[3], const void* vx,
          const void* vy, const void* vz, unsigned char* scratch, double* sums, dim3 grid) {
    constexpr double SMALL = 1.0e-50;
    std::memset(&P, 0, sizeof(P));
    P.nx = c.nx; P.ny = c.ny; P.nz = c.nz;
    P.pitch = c.nx; P.vxpitch = c.nx + 1; P.cpitch = c.nx;   // the caller's dense layouts
    P.plane = (long long)c.nx * c.ny;
    P.zsplit = (int)grid.z;
    P.zchunk = (c.nz + P.zsplit - 1) / P.zsplit;
    for (int k = 0; k < 3; ++k) {
        P.in[k] = static_cast<const T*>(in[k]);
        P.out[k] = static_cast<T*>(out[k]);
    }
    P.code = scratch + OFF_CODE;
    P.vx = static_cast<const T*>(vx);
    P.vy = static_cast<const T*>(vy);
    P.vz = static_cast<const T*>(vz);
    const double dTime = c.dt;
    P.hx = (T)(dTime / c.dx); P.hy = (T)(dTime / c.dy); P.hz = (T)(dTime / c.dz);
    P.hxx = (T)(dTime / (c.dx * c.dx)); P.hyy = (T)(dTime / (c.dy * c.dy)); P.hzz = (T)(dTime / (c.dz * c.dz));
    const double Bx = c.main_field[0], By = c.main_field[1], Bz = c.main_field[2];
    const double anb = std::sqrt(Bx * Bx + By * By + Bz * Bz);
    const double an[3] = {Bx / anb, By / anb, Bz / anb};
    for (int k = 0; k < 3; ++k) {
        P.an[k] = (T)an[k];
        P.peqn[k] = (T)(c.p_eq * an[k]);
    }
    P.b = (T)(dTime * c.gamma);
    P.dx = (T)c.dx; P.dy = (T)c.dy; P.dz = (T)c.dz;
    const double D = c.d_pore;
    P.dpp = (T)(2.0 * (D * D) / (D + D + SMALL));
    P.dps = (T)(2.0 * (SMALL * D) / (SMALL + D + SMALL));
    for (int f = 0; f < 64; ++f) {
        double ct1 = 1.0 / c.t1, ct2 = 1.0 / c.t2;
        const double d3[3] = {c.dx, c.dy, c.dz};
        for (int b = 0; b < 6; ++b)
            if (f & (1 << b)) {
                ct1 += c.rho1 / d3[b / 2];
                ct2 += c.rho2 / d3[b / 2];
            }
        P.dtt1[f] = (T)(dTime * (1.0 / (1.0 / ct1)));
        P.dtt2[f] = (T)(dTime * (1.0 / (1.0 / ct2)));
    }
    P.diffusion = c.diffusion ? 1 : 0;
    P.box[0] = c.buffer[0]; P.box[1] = c.nx - c.buffer[0];
    P.box[2] = c.buffer[1]; P.box[3] = c.ny - c.buffer[1];
    P.box[4] = c.buffer[2]; P.box[5] = c.nz - c.buffer[2];
    P.dxd = c.dx; P.dyd = c.dy; P.dzd = c.dz; P.gamma = c.gamma;
    P.steps = reinterpret_cast<const bt::StepInfo*>(scratch + OFF_STEP);
    P.nsched = 0;  // steps[0] is the record written by this call
    P.pulses = reinterpret_cast<const bt::DevPulse*>(scratch + OFF_PULSE);
    P.ctl = reinterpret_cast<bt::Ctl*>(scratch + OFF_CTL);
    P.partials = reinterpret_cast<double*>(scratch + OFF_PARTIALS);
    P.mt = sums;
    P.mt_cap = 1;
}

}  // namespace

extern "C" int bt_step_noalloc(const bt_config* cfg, const uint8_t* mask, const void* vx, const void* vy,
                               const void* vz, const void* mx_in, const void* my_in, const void* mz_in, void* mx_out,
                               void* my_out, void* mz_out, double* sums, void* stream) {
    if (!cfg || !mask || !mx_in || !my_in || !mz_in || !mx_out || !my_out || !mz_out || !sums) return BT_E_ARG;
    const bt_config& c = *cfg;
    if (c.scheme != BT_SCHEME_REFERENCE || (c.precision != BT_F32 && c.precision != BT_F64)) return BT_E_ARG;
    if (c.nx <= 0 || c.ny <= 0 || c.nz <= 0 || !(c.dt > 0) || !(c.dx > 0) || !(c.dy > 0) || !(c.dz > 0))
        return BT_E_ARG;
    for (int a = 0; a < 3; ++a)
        if (c.buffer[a] < 0 || 2 * c.buffer[a] > (a == 0 ? c.nx : a == 1 ? c.ny : c.nz)) return BT_E_ARG;
    // one field per call, advection on or off: a batched config (a q-sweep)
    // is not accepted, so no caller mistakes one stepped member for the batch
    if (c.batch > 1 || c.batch < 0 || (c.velocity != 0 && c.velocity != 1)) return BT_E_ARG;
    // a single step has no earlier step to have set non-copy ghost layers
    // (the first step of a run reads copies): copy faces only
    if (c.boundary[0] != BT_BC_COPY || c.boundary[1] != BT_BC_COPY || c.boundary[2] != BT_BC_COPY) return BT_E_ARG;
    if (c.velocity == 1 && (!vx || !vy || !vz)) return BT_E_ARG;
    const long long nvox = (long long)c.nx * c.ny * c.nz;
    if (nvox > BT_NOALLOC_MAX_VOXELS) {
        std::fprintf(stderr,
                     "bt_step_noalloc: %d x %d x %d = %lld voxels exceeds the allocation-free limit of %d voxels "
                     "(use bt_create / bt_run for larger grids)\n",
                     c.nx, c.ny, c.nz, nvox, BT_NOALLOC_MAX_VOXELS);
        return BT_E_SIZE;
    }
    // the generic kernel's grid: 32 x 8 column tiles, z split to fill the SMs,
    // no empty z-chunk
    const int gx = (c.nx + bt::TX - 1) / bt::TX, gy = (c.ny + bt::TY - 1) / bt::TY;
    const long long tiles = (long long)gx * gy;
    int zsplit = 1;
    if (tiles < 1216) zsplit = (int)std::min<long long>((1216 + tiles - 1) / tiles, std::max(1, c.nz / 8));
    zsplit = std::max(1, std::min(zsplit, c.nz));
    while ((c.nz + zsplit - 1) / zsplit > 1024) zsplit++;
    const int zchunk = (c.nz + zsplit - 1) / zsplit;
    zsplit = (c.nz + zchunk - 1) / zchunk;
    if (tiles * zsplit > BT_NOALLOC_MAX_BLOCKS) {
        std::fprintf(stderr, "bt_step_noalloc: grid of %lld blocks exceeds the allocation-free limit of %d\n",
                     tiles * zsplit, BT_NOALLOC_MAX_BLOCKS);
        return BT_E_SIZE;
    }
    const dim3 grid(gx, gy, zsplit);
    unsigned char* scratch = nullptr;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const cudaError_t se = scratch_for_current_device(s, &scratch);
    if (se == cudaErrorStreamCaptureUnsupported) {
        std::fprintf(stderr,
                     "bt_step_noalloc: the first call on a device looks up its scratch array and must come before "
                     "any stream capture\n");
        return BT_E_ARG;
    }
    if (se != cudaSuccess) return BT_E_CUDA;
    // the run-control block must start at zero (step 0, no ticket, no status)
    if (cudaMemsetAsync(scratch + OFF_CTL, 0, sizeof(bt::Ctl), s) != cudaSuccess) return BT_E_CUDA;
    noalloc_step_record_kernel<<<1, 32, 0, s>>>(reinterpret_cast<bt::StepInfo*>(scratch + OFF_STEP),
                                                reinterpret_cast<bt::DevPulse*>(scratch + OFF_PULSE), c.grad[0],
                                                c.grad[1], c.grad[2]);
    noalloc_code_kernel<<<1216, 256, 0, s>>>(mask, scratch + OFF_CODE, c.nx, c.ny, c.nz);
    if (cudaGetLastError() != cudaSuccess) return BT_E_CUDA;
    const void* in[3] = {mx_in, my_in, mz_in};
    void* out[3] = {mx_out, my_out, mz_out};
    const int prec = c.vector_mult == 1 ? 1 : 0;
    const int vel = c.velocity == 1 ? 1 : 0;
    cudaError_t e;
    if (c.precision == BT_F64) {
        bt::StepParams<double> P;
        fill<double>(c, P, in, out, vx, vy, vz, scratch, sums, grid);
        e = bt::launch_step<double>(P, BT_SCHEME_REFERENCE, vel, prec, grid, s);
    } else {
        bt::StepParams<float> P;
        fill<float>(c, P, in, out, vx, vy, vz, scratch, sums, grid);
        e = bt::launch_step<float>(P, BT_SCHEME_REFERENCE, vel, prec, grid, s);
    }
    return e == cudaSuccess ? BT_OK : BT_E_CUDA;
}
