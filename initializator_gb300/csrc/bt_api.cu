// Host runtime behind include/bt.h: handles, device memory, the per-step
// schedule table, kernel selection and the CUDA-graph-replayed step loop.
//
// Kernel selection per step: FP32 steps without pulses run the TMA fast path
// (bt_step_tma.cuh); FP64 steps and steps carrying pulses run the generic
// fused kernel (bt_step.cuh). Runs of GRAPH_STEPS pulse-free steps are
// replayed from a captured CUDA graph (the step index lives on the device).
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bt.h"
#include "bt_internal.h"

namespace {

constexpr double SMALL = 1.0e-50;
constexpr int GRAPH_STEPS = 32;   // steps per captured graph (even: the state returns to the same buffer)
constexpr int SUMS_BLOCKS = 1216; // 152 SMs x 8
constexpr int NUM_SMS_GB300 = 152;

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

}  // namespace

struct bt_handle {
    bt_config cfg{};
    int device = 0;
    int num_sms = NUM_SMS_GB300;
    cudaStream_t stream = nullptr;
    std::string err;
    size_t esz = 4;               // element size of the fields
    size_t nvox = 0;              // nx*ny*nz
    int pitch = 0, vxpitch = 0, cpitch = 0;
    size_t comp = 0;              // elements per component (pitch*ny*nz)
    int nb = 1;                   // fields advanced together (batch members)
    int gzsplit = 1;              // z-chunks per field, generic kernel
    int tzsplit = 1;              // z-chunks per tile column (at most), TMA kernel
    int tzlong = 0;               // tile columns with tzsplit chunks (the rest tzsplit - 1)
    int ttx = 128;                // tile width of the TMA kernel (128, or 64 for narrow grids)
    void* state_base[2] = {};     // one allocation per ping-pong side: [batch][component][z][y][pitch]
    void* state[2][3] = {};
    int cur = 0;
    uint8_t* code = nullptr;
    void* vel[3] = {};
    float* ucell = nullptr;       // fast path: gated cell velocities [axis][z][y][pitch]
    void* staging = nullptr;      // pinned host buffer: two halves of one component each (FP32 handles)
    size_t staging_bytes = 0;
    // staging slots of one component each: three (one per component, so a
    // field's upload never waits for its own copies, and one uploaded while
    // steps run returns once it is converted) up to 2^26 voxels, two above
    int nstage = 2;
    cudaEvent_t stage_ev[3] = {}; // the last copy through each slot
    // FP32 single fields with three staging slots: bt_set_state copies into
    // an inbox on a stream of its own (so the copy runs beside steps still
    // queued) and the handle's stream moves it into the field after them
    void* inbox = nullptr;
    bool no_inbox = false;        // no room for it on the device
    cudaStream_t xfer = nullptr;
    cudaEvent_t in_ready = nullptr, inbox_free = nullptr;
    bt::StepInfo* steps_d = nullptr;
    long long nsched = 0;
    std::vector<bt::StepInfo> steps_h;
    std::vector<double> kpos;     // wave vector at the start of each step (KSPACE): [step][batch][3]
    bt::DevPulse* pulses_d = nullptr;
    bt::Ctl* ctl_d = nullptr;
    bt::Ctl* ctl_h = nullptr;     // pinned
    double* partials_d = nullptr;
    size_t partials_cap = 0;
    size_t tpart = 0;             // fast path: doubles of partials per input side (two sides back to back)
    // fast path: the last step enqueued was a fast step whose partials wait
    // for the next fast step or a finish kernel (on input side fast_side)
    bool fast_pending = false;
    int fast_side = 0;
    double* mt_d = nullptr;
    long long mt_cap = 0;
    long long step = 0;
    long long last_run = 0;
    bool geometry = false;
    bool use_tma = false;
    dim3 grid;                    // generic kernel grid
    dim3 tgrid;                   // TMA kernel grid (zsplit, x tiles, y tiles)
    bt::StepParams<float> pf[2];
    bt::StepParams<double> pd[2];
    bt::StepParams<float> pt[2];  // TMA path (own z-chunking)
    bt::TmaMaps maps[2];
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_launches[2] = {0, 0};  // kernels one replay of each graph launches
    long long launches = 0;
    // per-voxel mode: [8][nz][ny][pitch] in the handle's precision: dTime/T1,
    // dTime/T2, then the face diffusivities -x +x -y +y -z +z
    void* fields_d = nullptr;
    // FP32 fast path with per-voxel rates: the rate palette (256 pairs of
    // dTime/T1, dTime/T2) and each voxel's index into it ([nz][ny][cpitch]);
    // pal_ok when the uploaded rates fit it (see bt_upload_rates)
    uint8_t* pal_idx = nullptr;
    float* pal_tab = nullptr;
    bool pal_ok = false;
    void* pred_base = nullptr;    // MacCormack predictor field [batch][component][z][y][pitch]
    // two-component sums: weights [2][nz][ny][pitch], block partials, M(t) x 6
    void* weights_d = nullptr;
    double* part6_d = nullptr;
    double* mt6_d = nullptr;
    long long mt6_cap = 0;
    std::vector<uint8_t> mask_h;  // host copy of the pore mask (two-component sums)
    uint32_t wait_polls = bt::RING_WAIT_POLLS;  // fast path's plane-ring wait bound
    int phase_axes = bt::PH_ALL;  // KSPACE: axes with a wave vector somewhere in the schedule
};

namespace {

int fail(bt_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

#define CK(h, call)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail(h, (e_ == cudaErrorMemoryAllocation) ? BT_E_NOMEM : BT_E_CUDA,               \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

void drop_graphs(bt_handle* h) {
    for (auto& g : h->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

// geometry code: bit f = in-domain solid face neighbour (-x,+x,-y,+y,-z,+z), bit 6 = pore
__global__ void code_kernel(const uint8_t* mask, uint8_t* code, int nx, int ny, int nz, int cpitch) {
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
        code[((long long)z * ny + y) * cpitch + x] = c;
    }
}

template <typename T>
void fill_params(bt_handle* h, bt::StepParams<T>* p, int zsplit, int zlong = 1 << 30) {
    const bt_config& c = h->cfg;
    const double dTime = c.dt;
    const double Bx = c.main_field[0], By = c.main_field[1], Bz = c.main_field[2];
    double an[3];
    if (c.scheme == BT_SCHEME_KSPACE) {
        an[0] = 0.0; an[1] = 0.0; an[2] = 1.0;
    } else {
        const double anb = std::sqrt(Bx * Bx + By * By + Bz * Bz);
        an[0] = Bx / anb; an[1] = By / anb; an[2] = Bz / anb;
    }
    const double D = c.d_pore;
    for (int s = 0; s < 2; ++s) {
        bt::StepParams<T>& P = p[s];
        std::memset(&P, 0, sizeof(P));
        P.nx = c.nx; P.ny = c.ny; P.nz = c.nz;
        P.pitch = h->pitch; P.vxpitch = h->vxpitch; P.cpitch = h->cpitch;
        P.plane = (long long)h->pitch * c.ny;
        P.zsplit = zsplit;
        P.zlong = zlong;
        P.zchunk = (c.nz + P.zsplit - 1) / P.zsplit;
        P.nbatch = h->nb;
        P.bstride = 3LL * (long long)h->comp;
        for (int k = 0; k < 3; ++k) {
            P.in[k] = static_cast<const T*>(h->state[s][k]);
            P.out[k] = static_cast<T*>(h->state[1 - s][k]);
        }
        P.code = h->code;
        P.vx = static_cast<const T*>(h->vel[0]);
        P.vy = static_cast<const T*>(h->vel[1]);
        P.vz = static_cast<const T*>(h->vel[2]);
        P.hx = (T)(dTime / c.dx); P.hy = (T)(dTime / c.dy); P.hz = (T)(dTime / c.dz);
        P.hxx = (T)(dTime / (c.dx * c.dx)); P.hyy = (T)(dTime / (c.dy * c.dy)); P.hzz = (T)(dTime / (c.dz * c.dz));
        for (int k = 0; k < 3; ++k) {
            P.an[k] = (T)an[k];
            P.peqn[k] = (T)(c.p_eq * an[k]);
        }
        P.b = (T)(dTime * c.gamma);
        P.dx = (T)c.dx; P.dy = (T)c.dy; P.dz = (T)c.dz;
        // ExplicitSimple regularises the harmonic mean with 1e-50, the GPU
        // MacCormack kernels with 1e-25
        const double reg = c.scheme == BT_SCHEME_MACCORMACK ? 1.0e-25 : SMALL;
        P.dpp = (T)(2.0 * (D * D) / (D + D + reg));
        P.dps = (T)(2.0 * (SMALL * D) / (SMALL + D + reg));
        // FillInDiffusinAndTime (cpp:1795-1841): bulk rate, then rho/d per solid
        // face in the order -x, +x, -y, +y, -z, +z; tau = 1/(1/rate) as ExplicitSimple reads it
        for (int f = 0; f < 64; ++f) {
            double ct1 = 1.0 / c.t1, ct2 = 1.0 / c.t2;
            const double d3[3] = {c.dx, c.dy, c.dz};
            for (int b = 0; b < 6; ++b)
                if (f & (1 << b)) {
                    ct1 += c.rho1 / d3[b / 2];
                    ct2 += c.rho2 / d3[b / 2];
                }
            const double tau1 = 1.0 / (1.0 / ct1), tau2 = 1.0 / (1.0 / ct2);
            P.dtt1[f] = (T)(dTime * tau1);
            P.dtt2[f] = (T)(dTime * tau2);
        }
        P.diffusion = c.diffusion ? 1 : 0;
        for (int a = 0; a < 3; ++a) P.bc[a] = c.boundary[a];
        P.box[0] = c.buffer[0]; P.box[1] = c.nx - c.buffer[0];
        P.box[2] = c.buffer[1]; P.box[3] = c.ny - c.buffer[1];
        P.box[4] = c.buffer[2]; P.box[5] = c.nz - c.buffer[2];
        P.dxd = c.dx; P.dyd = c.dy; P.dzd = c.dz; P.gamma = c.gamma;
        P.steps = h->steps_d;
        P.nsched = h->nsched;
        P.pulses = h->pulses_d;
        P.ctl = h->ctl_d;
        P.partials = h->partials_d;
        P.partials_prev = h->partials_d;
        P.side = s;
        P.mt = h->mt_d;
        P.mt_cap = h->mt_cap;
        P.fstride = (long long)h->comp;
        P.fdtt = h->fields_d ? static_cast<const T*>(h->fields_d) : nullptr;
        P.fw = h->fields_d ? static_cast<const T*>(h->fields_d) + 2 * h->comp : nullptr;
        P.pal = h->pal_ok ? h->pal_tab : nullptr;
        P.pal_idx = h->pal_ok ? h->pal_idx : nullptr;
        P.wait_polls = h->wait_polls;
        P.phase_axes = h->phase_axes;
    }
}

void refresh_params(bt_handle* h) {
    if (h->cfg.precision == BT_F64) {
        fill_params<double>(h, h->pd, h->gzsplit);
    } else {
        fill_params<float>(h, h->pf, h->gzsplit);
        fill_params<float>(h, h->pt, h->tzsplit, h->tzlong);
        // the fast path keeps one partials buffer per input side: a step's
        // partials are read by the next step, which writes the other buffer
        for (int s = 0; s < 2; ++s) {
            h->pt[s].partials = h->partials_d + s * h->tpart;
            h->pt[s].partials_prev = h->partials_d + (1 - s) * h->tpart;
        }
    }
    drop_graphs(h);
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

bool encode(CUtensorMap* m, CUtensorMapDataType t, int rank, void* base, const cuuint64_t* dims,
            const cuuint64_t* strides, const cuuint32_t* box) {
    auto fn = encoder();
    if (!fn) return false;
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return fn(m, t, rank, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// tensor maps of the FP32 fast path; false leaves the generic kernel in charge
bool build_maps(bt_handle* h) {
    const bt_config& c = h->cfg;
    const cuuint64_t nx = c.nx, ny = c.ny, nz = c.nz;
    const cuuint64_t P4 = (cuuint64_t)h->pitch * 4;
    for (int s = 0; s < 2; ++s) {
        bt::TmaMaps& M = h->maps[s];
        std::memset(&M, 0, sizeof(M));
        {
            cuuint64_t dims[5] = {nx, ny, nz, 3, (cuuint64_t)h->nb};
            cuuint64_t str[4] = {P4, P4 * ny, (cuuint64_t)h->comp * 4, (cuuint64_t)h->comp * 12};
            cuuint32_t box[5] = {(cuuint32_t)h->ttx + 8, (cuuint32_t)bt::tile_rows(h->ttx) + 2, 1, 3, 1};
            if (!encode(&M.state, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, h->state_base[s], dims, str, box)) return false;
        }
        {
            cuuint64_t dims[3] = {nx, ny, nz};
            cuuint64_t str[2] = {(cuuint64_t)h->cpitch, (cuuint64_t)h->cpitch * ny};
            cuuint32_t box[3] = {(cuuint32_t)h->ttx, (cuuint32_t)bt::tile_rows(h->ttx), 1};
            if (!encode(&M.code, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, h->code, dims, str, box)) return false;
        }
        if (h->pal_idx) {
            cuuint64_t dims[3] = {nx, ny, nz};
            cuuint64_t str[2] = {(cuuint64_t)h->cpitch, (cuuint64_t)h->cpitch * ny};
            cuuint32_t box[3] = {(cuuint32_t)h->ttx, (cuuint32_t)bt::tile_rows(h->ttx), 1};
            if (!encode(&M.pal, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, h->pal_idx, dims, str, box)) return false;
        }
        if (c.velocity == 1) {
            if (!h->ucell) return false;
            cuuint64_t dims[4] = {nx, ny, nz, 3};
            cuuint64_t str[3] = {P4, P4 * ny, (cuuint64_t)h->comp * 4};
            cuuint32_t box[4] = {(cuuint32_t)h->ttx, (cuuint32_t)bt::tile_rows(h->ttx), 1, 3};
            if (!encode(&M.ucell, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->ucell, dims, str, box)) return false;
        }
    }
    return true;
}

// z-chunking with no empty chunk: zsplit = ceil(nz / zchunk)
int normalise_split(int nz, int zsplit) {
    zsplit = std::max(1, std::min(zsplit, nz));
    while ((nz + zsplit - 1) / zsplit > 1024) zsplit++;
    const int zchunk = (nz + zsplit - 1) / zsplit;
    return (nz + zchunk - 1) / zchunk;
}

// tile columns of one field on the fast path
long long tma_tiles(const bt_handle* h) {
    const bt_config& c = h->cfg;
    const int tw = h->ttx, th = bt::tile_rows(tw);
    return (long long)((c.nx + tw - 1) / tw) * ((c.ny + th - 1) / th);
}

// the fast path's z-chunking: `chunks` chunks per field in total, spread over
// the tile columns so that they differ by at most one (at least one chunk per
// column, at most one plane per chunk, chunks of at most 1024 planes)
int set_tma_chunks(bt_handle* h, long long chunks) {
    const bt_config& c = h->cfg;
    const long long tiles = tma_tiles(h);
    const long long lo = tiles * ((c.nz + 1023) / 1024), hi = tiles * c.nz;
    chunks = std::max(lo, std::min(hi, chunks));
    const long long q = chunks / tiles, r = chunks % tiles;
    const int zsplit = (int)(r ? q + 1 : q), zlong = (int)(r ? r : tiles);
    // unchanged since the last call (tpart is only ever set here): keep the
    // captured graphs
    if (zsplit == h->tzsplit && zlong == h->tzlong && h->tpart > 0) return BT_OK;
    const int tw = h->ttx, th = bt::tile_rows(tw);
    const int gx = (c.nx + tw - 1) / tw, gy = (c.ny + th - 1) / th;
    h->tzsplit = zsplit;
    h->tzlong = zlong;
    h->tgrid = dim3(zsplit * h->nb, gx, gy);
    h->tpart = 3 * (size_t)zsplit * gx * gy * h->nb;
    const size_t need = 2 * h->tpart;
    if (need > h->partials_cap) {
        if (h->partials_d) cudaFree(h->partials_d);
        h->partials_d = nullptr;
        h->partials_cap = 0;
        CK(h, cudaMalloc(&h->partials_d, sizeof(double) * need));
        h->partials_cap = need;
    }
    refresh_params(h);
    return BT_OK;
}

// the same number of chunks in every tile column
int set_tma_split(bt_handle* h, int zsplit) {
    return set_tma_chunks(h, (long long)normalise_split(h->cfg.nz, zsplit) * tma_tiles(h));
}

// default split: about 4 waves of 2 CTAs per SM, chunks of at least 8 planes
int default_tma_split(const bt_handle* h) {
    const bt_config& c = h->cfg;
    const int tw = h->ttx, th = bt::tile_rows(tw);
    const long long tiles = (long long)((c.nx + tw - 1) / tw) * ((c.ny + th - 1) / th) * h->nb;
    const long long slots = 2LL * h->num_sms;
    long long zs = (4 * slots + tiles - 1) / tiles;
    zs = std::min<long long>(zs, std::max(1, c.nz / 8));
    if (const char* e = std::getenv("BT_TMA_ZSPLIT")) zs = std::max(1, std::atoi(e));
    return (int)std::max<long long>(1, zs);
}

// the FP32 fast path serves this configuration (non-copy faces: KSPACE only)
bool fast_path_config(const bt_config& c) {
    if (c.precision != BT_F32 || c.scheme == BT_SCHEME_MACCORMACK || std::getenv("BT_NO_TMA")) return false;
    return c.scheme == BT_SCHEME_KSPACE ||
           (c.boundary[0] == BT_BC_COPY && c.boundary[1] == BT_BC_COPY && c.boundary[2] == BT_BC_COPY);
}

bool step_has_pulse(const bt_handle* h, long long s) {
    return s < h->nsched && h->steps_h[s * h->nb].pulse_count > 0;
}

// close a run of fast steps: the finish kernel adds the last step's partials
// and brings Ctl::step up to date (a no-op when nothing is pending)
cudaError_t finish_fast(bt_handle* h) {
    if (!h->fast_pending) return cudaSuccess;
    h->fast_pending = false;
    h->launches++;
    return bt::launch_tma_finish(h->pt[h->fast_side], h->tgrid, h->stream);
}

cudaError_t launch_one(bt_handle* h, int side, long long abs_step) {
    const bt_config& c = h->cfg;
    const int prec = (c.scheme != BT_SCHEME_KSPACE && c.vector_mult == 1) ? 1 : 0;
    const int vel = c.velocity == 1 ? 1 : 0;
    // a pulse step runs on the fast path when all its pulses are fixed-angle
    // (one rotation; not with the rate palette)
    const bool pulse = step_has_pulse(h, abs_step);
    const bool fast = c.precision == BT_F32 && c.scheme != BT_SCHEME_MACCORMACK && h->use_tma && !h->fields_d &&
                      (!pulse || (!h->pal_ok && h->steps_h[abs_step * h->nb].rot_ok));
    cudaError_t e;
    if (fast) {
        // a fast step after a fast step adds its predecessor's partials
        h->launches++;
        e = bt::launch_step_tma(h->pt[side], h->maps[side], c.scheme, vel, prec, h->pal_ok, pulse, h->tgrid,
                                h->ttx, !h->fast_pending, h->stream);
        h->fast_pending = true;
        h->fast_side = side;
        // the two-component sums read Ctl::step
        if (e == cudaSuccess && h->weights_d) e = finish_fast(h);
    } else {
        e = finish_fast(h);
        if (e != cudaSuccess) return e;
        h->launches++;
        if (c.scheme == BT_SCHEME_MACCORMACK) {
            h->launches++;  // predictor + corrector
            char* pb = static_cast<char*>(h->pred_base);
            if (c.precision == BT_F64) {
                double* pr[3] = {(double*)pb, (double*)(pb + 8 * h->comp), (double*)(pb + 16 * h->comp)};
                e = bt::launch_mac<double>(h->pd[side], pr, vel, prec, h->grid, h->stream);
            } else {
                float* pr[3] = {(float*)pb, (float*)(pb + 4 * h->comp), (float*)(pb + 8 * h->comp)};
                e = bt::launch_mac<float>(h->pf[side], pr, vel, prec, h->grid, h->stream);
            }
        } else if (c.precision == BT_F64)
            e = bt::launch_step<double>(h->pd[side], c.scheme, vel, prec, h->grid, h->stream);
        else
            e = bt::launch_step<float>(h->pf[side], c.scheme, vel, prec, h->grid, h->stream);
    }
    if (e != cudaSuccess || !h->weights_d) return e;
    // two-component sums of the field this step wrote
    h->launches += 2;
    if (c.precision == BT_F64) {
        const double* w = static_cast<const double*>(h->weights_d);
        return bt::launch_phase_sums<double>(h->pd[side], w, w + h->comp, h->part6_d, SUMS_BLOCKS, h->mt6_d,
                                             h->mt6_cap, h->stream);
    }
    const float* w = static_cast<const float*>(h->weights_d);
    return bt::launch_phase_sums<float>(h->pf[side], w, w + h->comp, h->part6_d, SUMS_BLOCKS, h->mt6_d, h->mt6_cap,
                                        h->stream);
}

// per-step table: gradient, KSPACE wave vector and face phases, pulse ranges
int build_schedule(bt_handle* h, const bt_pulse* pulses, int npulses, const double* grad_wave, long long nwave) {
    const bt_config& c = h->cfg;
    long long nsched = std::max<long long>(nwave, 0);
    for (int q = 0; q < npulses; ++q) {
        if (pulses[q].step < 0) return fail(h, BT_E_ARG, "pulse with a negative step");
        if (c.scheme == BT_SCHEME_KSPACE && pulses[q].flag != 2)
            return fail(h, BT_E_ARG, "the KSPACE scheme takes RF pulses (flag 2) only; gradients go in the waveform");
        if (pulses[q].flag < 1 || pulses[q].flag > 4) return fail(h, BT_E_ARG, "pulse flag must be 1..4");
        nsched = std::max(nsched, pulses[q].step + 1);
    }
    std::vector<int> order(npulses);
    for (int q = 0; q < npulses; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pulses[a].step < pulses[b].step; });
    std::vector<bt::DevPulse> dp(std::max(npulses, 1));
    for (int q = 0; q < npulses; ++q) {
        const bt_pulse& p = pulses[order[q]];
        bt::DevPulse& d = dp[q];
        std::memset(&d, 0, sizeof(d));
        d.flag = p.flag;
        d.param = p.param;
        const double nx = p.axis[0], ny = p.axis[1], nz = p.axis[2];
        double length = std::pow(nx * nx + ny * ny + nz * nz, 0.5);  // AddImpulse, cpp:2558-2564
        if (length == 0.0) length = 1.0;
        for (int k = 0; k < 3; ++k) d.axis[k] = p.axis[k];
        d.naxis[0] = nx / length; d.naxis[1] = ny / length; d.naxis[2] = nz / length;
        d.eff = std::pow(nx * nx + ny * ny + nz * nz, 0.5);
    }
    // one record per step and batch member ([step][member]); grad_wave is
    // [nwave][member][3]; the members share the pulses
    const int nb = h->nb;
    std::vector<bt::StepInfo> st((nsched + 1) * nb);
    h->kpos.assign(3 * (nsched + 1) * nb, 0.0);
    const double d3[3] = {c.dx, c.dy, c.dz};
    for (int b = 0; b < nb; ++b) {
        double k[3] = {0.0, 0.0, 0.0};
        int qi = 0;
        for (long long s = 0; s <= nsched; ++s) {
            bt::StepInfo& si = st[s * nb + b];
            std::memset(&si, 0, sizeof(si));
            const bool in_wave = grad_wave && s < nwave;
            for (int a = 0; a < 3; ++a) si.grad[a] = in_wave ? grad_wave[3 * (s * nb + b) + a] : c.grad[a];
            if (s == nsched)  // the default entry used beyond the table: cfg gradient, no pulses
                for (int a = 0; a < 3; ++a) si.grad[a] = c.grad[a];
            for (int a = 0; a < 3; ++a) h->kpos[3 * (s * nb + b) + a] = k[a];
            // KSPACE: the stencil acts at the middle of the step (half the
            // step's precession, the stencil, the other half): a precession
            // only moves the frame and leaves the stored values alone, so this
            // symmetric split costs nothing but taking the face phases at
            // k + gamma G dt / 2, and makes the gradient dephasing of the step
            // second order in dt (the k at its start would make it first order)
            double km[3] = {k[0], k[1], k[2]};
            if (c.scheme == BT_SCHEME_KSPACE && s < nsched)
                for (int a = 0; a < 3; ++a) km[a] = k[a] + 0.5 * (c.gamma * si.grad[a] * c.dt);
            for (int a = 0; a < 3; ++a) {
                // neighbour at -d: exp(+i k d); at +d: exp(-i k d)
                const double ang = km[a] * d3[a];
                si.phase[2 * a][0] = std::cos(ang);
                si.phase[2 * a][1] = std::sin(ang);
                si.phase[2 * a + 1][0] = std::cos(ang);
                si.phase[2 * a + 1][1] = -std::sin(ang);
                si.phasef[a][0] = (float)si.phase[2 * a][0];
                si.phasef[a][1] = (float)si.phase[2 * a][1];
                // periodic faces: exp(-i k_a n_a d_a), the far edge cell's
                // k-frame value moved across the period
                const int n3[3] = {c.nx, c.ny, c.nz};
                const double wa = km[a] * ((double)n3[a] * d3[a]);
                si.wrap[a][0] = std::cos(wa);
                si.wrap[a][1] = -std::sin(wa);
                si.wrapf[a][0] = (float)si.wrap[a][0];
                si.wrapf[a][1] = (float)si.wrap[a][1];
            }
            if (c.scheme == BT_SCHEME_KSPACE && s < nsched)
                for (int a = 0; a < 3; ++a) k[a] = k[a] + c.gamma * si.grad[a] * c.dt;
            for (int a = 0; a < 3; ++a) si.knext[a] = k[a];
            si.pulse_first = qi;
            while (qi < npulses && pulses[order[qi]].step == s) qi++;
            si.pulse_count = s < nsched ? qi - si.pulse_first : 0;
            if (si.pulse_count > 0) {
                // all fixed-angle: the FP32 fast path applies their product
                double r[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
                bool fixed = true;
                for (int q = si.pulse_first; fixed && q < si.pulse_first + si.pulse_count; ++q) {
                    fixed = dp[q].flag == 2;
                    if (fixed) bt::fixed_pulse_then(std::cos(dp[q].param), std::sin(dp[q].param), dp[q].axis, r);
                }
                si.rot_ok = fixed ? 1 : 0;
                for (int i = 0; i < 9; ++i) si.rotf[i] = (float)r[i];
            }
        }
    }
    if (h->steps_d) cudaFree(h->steps_d);
    if (h->pulses_d) cudaFree(h->pulses_d);
    h->steps_d = nullptr;
    h->pulses_d = nullptr;
    CK(h, cudaMalloc(&h->steps_d, sizeof(bt::StepInfo) * st.size()));
    CK(h, cudaMalloc(&h->pulses_d, sizeof(bt::DevPulse) * dp.size()));
    CK(h, cudaMemcpy(h->steps_d, st.data(), sizeof(bt::StepInfo) * st.size(), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->pulses_d, dp.data(), sizeof(bt::DevPulse) * dp.size(), cudaMemcpyHostToDevice));
    h->steps_h.swap(st);
    h->nsched = nsched;
    // the axes along which some step's wave vector (at its start or end) is
    // not zero: the fast path drops the face phases of the others exactly
    bool kxy = false, kz = false;
    for (size_t q = 0; q < h->kpos.size(); q += 3) {
        kxy = kxy || h->kpos[q] != 0.0 || h->kpos[q + 1] != 0.0;
        kz = kz || h->kpos[q + 2] != 0.0;
    }
    h->phase_axes = kxy ? bt::PH_ALL : (kz ? bt::PH_Z : bt::PH_NONE);
    refresh_params(h);
    return BT_OK;
}

void kvec_at(const bt_handle* h, long long s, int b, double k[3]) {
    if (h->cfg.scheme != BT_SCHEME_KSPACE || h->kpos.empty()) {
        k[0] = k[1] = k[2] = 0.0;
        return;
    }
    const long long i = std::min<long long>(s, h->nsched);
    for (int a = 0; a < 3; ++a) k[a] = h->kpos[3 * (i * h->nb + b) + a];
}

int ensure_mt(bt_handle* h, long long n) {
    if (h->weights_d && n > h->mt6_cap) {
        const long long cap = std::max<long long>(n, 1024);
        if (h->mt6_d) cudaFree(h->mt6_d);
        h->mt6_d = nullptr;
        h->mt6_cap = 0;
        drop_graphs(h);  // captured launches hold the old buffer
        CK(h, cudaMalloc(&h->mt6_d, sizeof(double) * 6 * cap));
        h->mt6_cap = cap;
    }
    if (n <= h->mt_cap) return BT_OK;
    long long cap = std::max<long long>(n, 1024);
    if (h->mt_d) cudaFree(h->mt_d);
    h->mt_d = nullptr;
    h->mt_cap = 0;
    CK(h, cudaMalloc(&h->mt_d, sizeof(double) * 3 * cap * h->nb));
    h->mt_cap = cap;
    refresh_params(h);
    return BT_OK;
}

int check_ctl(bt_handle* h) {
    CK(h, cudaMemcpyAsync(h->ctl_h, h->ctl_d, sizeof(bt::Ctl), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->ctl_h->status & 8) return fail(h, BT_E_TIMEOUT, "a bounded device wait (TMA mbarrier) gave up");
    if (h->ctl_h->step != h->step)
        return fail(h, BT_E_STATE, "device step counter " + std::to_string(h->ctl_h->step) + " != host " +
                                       std::to_string(h->step));
    if (h->ctl_h->status & 4) return fail(h, BT_E_NAN, "M(t) watchdog: a sum is NaN or Inf");
    if (h->ctl_h->status & 1) return fail(h, BT_E_STATE, "M(t) buffer overflow");
    return BT_OK;
}

// (x + i y) of every member's field *= exp(sign * i * k_member . r) at the current step
int frame_change(bt_handle* h, void* const* f, int sign) {
    const bt_config& c = h->cfg;
    for (int b = 0; b < h->nb; ++b) {
        double k[3];
        kvec_at(h, h->step, b, k);
        if (k[0] == 0.0 && k[1] == 0.0 && k[2] == 0.0) continue;
        const size_t off = (size_t)b * 3 * h->comp * h->esz;
        cudaError_t e;
        if (h->esz == 8) {
            double* fp[3] = {(double*)((char*)f[0] + off), (double*)((char*)f[1] + off), (double*)((char*)f[2] + off)};
            e = bt::launch_frame<double>(fp, h->code, c.nx, c.ny, c.nz, h->pitch, h->cpitch, k[0], k[1], k[2], c.dx,
                                         c.dy, c.dz, sign, h->stream);
        } else {
            float* fp[3] = {(float*)((char*)f[0] + off), (float*)((char*)f[1] + off), (float*)((char*)f[2] + off)};
            e = bt::launch_frame<float>(fp, h->code, c.nx, c.ny, c.nz, h->pitch, h->cpitch, k[0], k[1], k[2], c.dx,
                                        c.dy, c.dz, sign, h->stream);
        }
        CK(h, e);
        h->launches++;
    }
    return BT_OK;
}

bool any_phase(const bt_handle* h) {
    for (int b = 0; b < h->nb; ++b) {
        double k[3];
        kvec_at(h, h->step, b, k);
        if (k[0] != 0.0 || k[1] != 0.0 || k[2] != 0.0) return true;
    }
    return false;
}

// fn(a, b) over the slices [a, b) of [0, n), on up to 32 of the host's
// cores with at least `grain` items each (on the calling thread alone when n
// is small)
template <typename F>
void parallel_slices(size_t n, size_t grain, F fn) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::max<size_t>(1, std::min<size_t>(std::min(hw, 32u), n / std::max<size_t>(1, grain)));
    auto part = [&fn, n, nt](unsigned t) { fn(n * t / nt, n * (t + 1) / nt); };
    if (nt == 1) {
        part(0);
        return;
    }
    // a thread that cannot be started (a process limit) leaves its slice to
    // the calling thread: no exception crosses the C ABI
    std::vector<std::thread> ts;
    ts.reserve(nt - 1);
    std::vector<unsigned> left;
    for (unsigned t = 1; t < nt; ++t) {
        try {
            ts.emplace_back(part, t);
        } catch (...) {
            left.push_back(t);
        }
    }
    part(0);
    for (unsigned t : left) part(t);
    for (auto& t : ts) t.join();
}

// Pinned staging buffers of destroyed handles, kept for the next handle on
// the same device (pinning hundreds of MB costs tens of ms, as much as a
// short solve); a handle takes the smallest kept buffer that is large
// enough. At most PINNED_KEEP bytes are kept; the rest are freed.
constexpr size_t PINNED_KEEP = (size_t)2 << 30;
std::mutex g_pinned_mu;
struct Pinned {
    int device;
    size_t bytes;
    void* p;
};
std::vector<Pinned> g_pinned;

cudaError_t pinned_get(int device, size_t bytes, void** out) {
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        int best = -1;
        for (int i = 0; i < (int)g_pinned.size(); ++i)
            if (g_pinned[i].device == device && g_pinned[i].bytes >= bytes &&
                (best < 0 || g_pinned[i].bytes < g_pinned[best].bytes))
                best = i;
        if (best >= 0) {
            *out = g_pinned[best].p;
            g_pinned.erase(g_pinned.begin() + best);
            return cudaSuccess;
        }
    }
    return cudaMallocHost(out, bytes);
}

void pinned_put(int device, size_t bytes, void* p) {
    std::vector<void*> drop;
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        g_pinned.push_back({device, bytes, p});
        size_t total = 0;
        for (const Pinned& b : g_pinned) total += b.bytes;
        // free the oldest beyond the bound
        while (total > PINNED_KEEP && !g_pinned.empty()) {
            total -= g_pinned.front().bytes;
            drop.push_back(g_pinned.front().p);
            g_pinned.erase(g_pinned.begin());
        }
    }
    for (void* q : drop) cudaFreeHost(q);
}

// dense [nz][ny][nx] host component <-> pitched device component
// dst[q] = src[q] (a precision conversion) for q < n, over the host's cores
// when the field is large, so that the host side of a transfer keeps up with
// the copy engine
template <typename D, typename S>
void convert(D* dst, const S* src, size_t n) {
    parallel_slices(n, (size_t)1 << 20, [dst, src](size_t a, size_t b) {
        for (size_t q = a; q < b; ++q) dst[q] = (D)src[q];
    });
}

// host FP64 component -> device field. FP32 handles convert into staging slot
// `half` (once the previous copy out of it has finished) and copy from there,
// so consecutive components take consecutive slots and each conversion
// overlaps the previous component's copy
int put_component(bt_handle* h, void* dst, const double* src, int half, cudaStream_t s) {
    const bt_config& c = h->cfg;
    const size_t rows = (size_t)c.ny * c.nz;
    if (h->esz == 8) {
        CK(h, cudaMemcpy2DAsync(dst, h->pitch * 8, src, c.nx * 8, c.nx * 8, rows, cudaMemcpyHostToDevice, s));
    } else {
        float* f = static_cast<float*>(h->staging) + (size_t)half * h->nvox;
        CK(h, cudaEventSynchronize(h->stage_ev[half]));
        convert(f, src, h->nvox);
        CK(h, cudaMemcpy2DAsync(dst, h->pitch * 4, f, c.nx * 4, c.nx * 4, rows, cudaMemcpyHostToDevice, s));
        CK(h, cudaEventRecord(h->stage_ev[half], s));
    }
    return BT_OK;
}

// device field components -> host FP64 (n of them): for FP32 handles the copy
// of component i + 1 into one staging half runs while component i is
// converted out of the other
int get_components(bt_handle* h, double* const* dst, const void* const* src, int n) {
    const bt_config& c = h->cfg;
    const size_t rows = (size_t)c.ny * c.nz;
    if (h->esz == 8) {
        for (int i = 0; i < n; ++i)
            CK(h, cudaMemcpy2DAsync(dst[i], c.nx * 8, src[i], h->pitch * 8, c.nx * 8, rows, cudaMemcpyDeviceToHost,
                                    h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        return BT_OK;
    }
    float* f = static_cast<float*>(h->staging);
    for (int i = 0; i <= n; ++i) {
        if (i < n) {
            // the half was last read by the conversion of component i - 2, done by now
            float* fi = f + (size_t)(i & 1) * h->nvox;
            CK(h, cudaMemcpy2DAsync(fi, c.nx * 4, src[i], h->pitch * 4, c.nx * 4, rows, cudaMemcpyDeviceToHost,
                                    h->stream));
            CK(h, cudaEventRecord(h->stage_ev[i & 1], h->stream));
        }
        if (i > 0) {
            const int j = i - 1;
            CK(h, cudaEventSynchronize(h->stage_ev[j & 1]));
            convert(dst[j], f + (size_t)(j & 1) * h->nvox, h->nvox);
        }
    }
    return BT_OK;
}

}  // namespace

extern "C" {

const char* bt_version(void) { return "initializator_gb300 0.2 (sm_103a)"; }

int bt_create(const bt_config* cfg, bt_handle** out) {
    if (!cfg || !out) return BT_E_ARG;
    *out = nullptr;
    if (cfg->nx <= 0 || cfg->ny <= 0 || cfg->nz <= 0) return BT_E_ARG;
    if (cfg->precision != BT_F32 && cfg->precision != BT_F64) return BT_E_ARG;
    if (cfg->scheme != BT_SCHEME_REFERENCE && cfg->scheme != BT_SCHEME_KSPACE && cfg->scheme != BT_SCHEME_MACCORMACK)
        return BT_E_ARG;
    if (!(cfg->dt > 0) || !(cfg->dx > 0) || !(cfg->dy > 0) || !(cfg->dz > 0)) return BT_E_ARG;
    for (int a = 0; a < 3; ++a)
        if (cfg->buffer[a] < 0 || 2 * cfg->buffer[a] > (a == 0 ? cfg->nx : a == 1 ? cfg->ny : cfg->nz)) return BT_E_ARG;
    for (int a = 0; a < 3; ++a)
        if (cfg->boundary[a] != BT_BC_COPY && cfg->boundary[a] != BT_BC_PERIODIC && cfg->boundary[a] != BT_BC_ZERO)
            return BT_E_ARG;
    const long long nvox = (long long)cfg->nx * cfg->ny * cfg->nz;
    if (nvox > (1LL << 40) || cfg->nx > (1 << 28) || cfg->ny > (1 << 28)) return BT_E_ARG;
    bt_handle* h = new bt_handle();
    h->cfg = *cfg;
    h->esz = cfg->precision == BT_F64 ? 8 : 4;
    h->nvox = (size_t)nvox;
    h->pitch = round_up(cfg->nx, 4);
    h->vxpitch = round_up(cfg->nx + 1, 4);
    h->cpitch = round_up(cfg->nx, 16);
    h->comp = (size_t)h->pitch * cfg->ny * cfg->nz;
    h->nb = cfg->batch > 1 ? cfg->batch : 1;
    int rc = BT_OK;
    auto bail = [&](int code) {
        bt_destroy(h);
        return code;
    };
    if (cudaGetDevice(&h->device) != cudaSuccess) return bail(BT_E_CUDA);
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(BT_E_CUDA);
    // generic kernel grid: 32 x 8 column tiles; z split so that the grid fills the SMs several times
    const int gx = (cfg->nx + bt::TX - 1) / bt::TX, gy = (cfg->ny + bt::TY - 1) / bt::TY;
    int zsplit = 1;
    const long long tiles = (long long)gx * gy * h->nb;
    const long long want = 8LL * h->num_sms;
    if (tiles < want) zsplit = (int)std::min<long long>((want + tiles - 1) / tiles, std::max(1, cfg->nz / 8));
    if (const char* e = std::getenv("BT_ZSPLIT")) zsplit = std::max(1, std::atoi(e));
    zsplit = normalise_split(cfg->nz, zsplit);
    h->gzsplit = zsplit;
    h->grid = dim3(gx, gy, zsplit * h->nb);  // blockIdx.z = z-chunk + zsplit * batch member
    const size_t sbytes = 3 * h->esz * h->comp * h->nb;
    for (int s = 0; s < 2; ++s) {
        if (cudaMalloc(&h->state_base[s], sbytes) != cudaSuccess) return bail(BT_E_NOMEM);
        cudaMemset(h->state_base[s], 0, sbytes);
        for (int k = 0; k < 3; ++k) h->state[s][k] = static_cast<char*>(h->state_base[s]) + k * h->esz * h->comp;
    }
    if (cfg->scheme == BT_SCHEME_MACCORMACK) {
        // the predictor's field (zero in solid, as the reference's memset)
        if (cudaMalloc(&h->pred_base, sbytes) != cudaSuccess) return bail(BT_E_NOMEM);
        cudaMemset(h->pred_base, 0, sbytes);
    }
    const size_t cbytes = (size_t)h->cpitch * cfg->ny * cfg->nz;
    if (cudaMalloc(&h->code, cbytes) != cudaSuccess) return bail(BT_E_NOMEM);
    cudaMemset(h->code, 0, cbytes);
    if (cfg->velocity == 1) {
        const size_t n3[3] = {(size_t)h->vxpitch * cfg->ny * cfg->nz, (size_t)h->pitch * (cfg->ny + 1) * cfg->nz,
                              (size_t)h->pitch * cfg->ny * (cfg->nz + 1)};
        for (int a = 0; a < 3; ++a) {
            if (cudaMalloc(&h->vel[a], h->esz * n3[a]) != cudaSuccess) return bail(BT_E_NOMEM);
            cudaMemset(h->vel[a], 0, h->esz * n3[a]);
        }
        if (fast_path_config(*cfg)) {
            if (cudaMalloc(&h->ucell, sizeof(float) * 3 * h->comp) != cudaSuccess) return bail(BT_E_NOMEM);
            cudaMemset(h->ucell, 0, sizeof(float) * 3 * h->comp);
        }
    }
    if (cfg->precision == BT_F32) {
        h->nstage = h->nvox <= ((size_t)1 << 26) ? 3 : 2;
        h->staging_bytes = (size_t)h->nstage * 4 * h->nvox;
        if (pinned_get(h->device, h->staging_bytes, &h->staging) != cudaSuccess) {
            h->staging = nullptr;
            return bail(BT_E_NOMEM);
        }
        for (auto& e : h->stage_ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bail(BT_E_CUDA);
    }
    if (cfg->batch < 0 || (long long)h->nb * (long long)h->comp * 3 > (1LL << 40)) return bail(BT_E_ARG);
    const size_t nblocks = (size_t)h->grid.x * h->grid.y * h->grid.z;
    h->partials_cap = std::max<size_t>(3 * nblocks, 4 * SUMS_BLOCKS);
    if (cudaMalloc(&h->partials_d, sizeof(double) * h->partials_cap) != cudaSuccess) return bail(BT_E_NOMEM);
    if (cudaMalloc(&h->ctl_d, sizeof(bt::Ctl)) != cudaSuccess) return bail(BT_E_NOMEM);
    if (cudaMallocHost(&h->ctl_h, sizeof(bt::Ctl)) != cudaSuccess) return bail(BT_E_NOMEM);
    std::memset(h->ctl_h, 0, sizeof(bt::Ctl));
    if (cudaMemcpy(h->ctl_d, h->ctl_h, sizeof(bt::Ctl), cudaMemcpyHostToDevice) != cudaSuccess) return bail(BT_E_CUDA);
    h->tgrid = dim3(1, 1, 1);
    rc = ensure_mt(h, 1024);
    if (rc) return bail(rc);
    rc = build_schedule(h, nullptr, 0, nullptr, 0);
    if (rc) return bail(rc);
    if (fast_path_config(*cfg)) {
        // 64-wide tiles where they pad x less than 128-wide ones (narrow or
        // odd widths); BT_TMA_TW = 64 / 128 forces one
        h->ttx = ((cfg->nx + 63) / 64) * 64 < ((cfg->nx + 127) / 128) * 128 ? 64 : 128;
        if (const char* e = std::getenv("BT_TMA_TW")) h->ttx = std::atoi(e) == 64 ? 64 : 128;
        rc = set_tma_split(h, default_tma_split(h));
        if (rc) return bail(rc);
    }
    *out = h;
    return BT_OK;
}

int bt_destroy(bt_handle* h) {
    if (!h) return BT_OK;
    drop_graphs(h);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->xfer) cudaStreamSynchronize(h->xfer);  // its copies read the staging buffer
    for (auto& p : h->state_base)
        if (p) cudaFree(p);
    for (auto& p : h->vel)
        if (p) cudaFree(p);
    if (h->ucell) cudaFree(h->ucell);
    if (h->code) cudaFree(h->code);
    if (h->steps_d) cudaFree(h->steps_d);
    if (h->pulses_d) cudaFree(h->pulses_d);
    if (h->ctl_d) cudaFree(h->ctl_d);
    if (h->ctl_h) cudaFreeHost(h->ctl_h);
    if (h->staging) pinned_put(h->device, h->staging_bytes, h->staging);
    for (auto& e : h->stage_ev)
        if (e) cudaEventDestroy(e);
    if (h->partials_d) cudaFree(h->partials_d);
    if (h->mt_d) cudaFree(h->mt_d);
    if (h->fields_d) cudaFree(h->fields_d);
    if (h->pal_idx) cudaFree(h->pal_idx);
    if (h->pal_tab) cudaFree(h->pal_tab);
    if (h->pred_base) cudaFree(h->pred_base);
    if (h->weights_d) cudaFree(h->weights_d);
    if (h->part6_d) cudaFree(h->part6_d);
    if (h->mt6_d) cudaFree(h->mt6_d);
    if (h->xfer) cudaStreamDestroy(h->xfer);
    if (h->in_ready) cudaEventDestroy(h->in_ready);
    if (h->inbox_free) cudaEventDestroy(h->inbox_free);
    if (h->inbox) cudaFree(h->inbox);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return BT_OK;
}

const char* bt_last_error(const bt_handle* h) { return h ? h->err.c_str() : "null handle"; }

int bt_upload_geometry(bt_handle* h, const uint8_t* mask, const double* vx, const double* vy, const double* vz) {
    if (!h || !mask) return fail(h, BT_E_ARG, "mask is required");
    const bt_config& c = h->cfg;
    if (c.velocity == 1 && (!vx || !vy || !vz)) return fail(h, BT_E_ARG, "velocity == 1 needs vx, vy and vz");
    h->mask_h.assign(mask, mask + h->nvox);
    // per-voxel rates belong to the geometry they were uploaded with
    if (h->fields_d || h->pal_ok) {
        CK(h, cudaStreamSynchronize(h->stream));
        if (h->fields_d) cudaFree(h->fields_d);
        h->fields_d = nullptr;
        h->pal_ok = false;
    }
    uint8_t* mtmp = nullptr;
    CK(h, cudaMalloc(&mtmp, h->nvox));
    cudaError_t e = cudaMemcpy(mtmp, mask, h->nvox, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        code_kernel<<<1216, 256, 0, h->stream>>>(mtmp, h->code, c.nx, c.ny, c.nz, h->cpitch);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    cudaFree(mtmp);
    CK(h, e);
    if (c.velocity == 1) {
        // dense [k][j][i] faces -> pitched rows
        const int w3[3] = {c.nx + 1, c.nx, c.nx};
        const int p3[3] = {h->vxpitch, h->pitch, h->pitch};
        const size_t rows3[3] = {(size_t)c.ny * c.nz, (size_t)(c.ny + 1) * c.nz, (size_t)c.ny * (c.nz + 1)};
        const double* src[3] = {vx, vy, vz};
        for (int a = 0; a < 3; ++a) {
            const size_t n = (size_t)w3[a] * rows3[a];
            if (h->esz == 8) {
                CK(h, cudaMemcpy2D(h->vel[a], p3[a] * 8, src[a], w3[a] * 8, w3[a] * 8, rows3[a], cudaMemcpyHostToDevice));
            } else {
                std::vector<float> f(n);
                convert(f.data(), src[a], n);
                CK(h, cudaMemcpy2D(h->vel[a], p3[a] * 4, f.data(), w3[a] * 4, w3[a] * 4, rows3[a],
                                   cudaMemcpyHostToDevice));
            }
        }
        if (h->ucell) {
            CK(h, bt::launch_cell_velocity(h->pt[0], h->ucell, (long long)h->comp, h->stream));
            CK(h, cudaStreamSynchronize(h->stream));
        }
    }
    h->geometry = true;
    if (fast_path_config(h->cfg) && h->tgrid.y > 0) h->use_tma = build_maps(h);
    refresh_params(h);
    return BT_OK;
}

int bt_set_state(bt_handle* h, const double* mx, const double* my, const double* mz) {
    if (!h || !mx || !my || !mz) return fail(h, BT_E_ARG, "null field");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    const double* src[3] = {mx, my, mz};
    bool use_inbox = h->esz == 4 && h->nb == 1 && h->nstage == 3 && !h->no_inbox;
    if (use_inbox && !h->inbox && cudaMalloc(&h->inbox, 3 * h->comp * 4) != cudaSuccess) {
        // the inbox only overlaps copies with steps: without room for it the
        // copies go straight into the field
        cudaGetLastError();
        h->inbox = nullptr;
        h->no_inbox = true;
        use_inbox = false;
    }
    if (use_inbox) {
        // through the inbox: the host-to-device copies run on the transfer
        // stream beside any steps still queued, then one device copy moves
        // the field in after them
        if (!h->xfer) {
            CK(h, cudaMemset(h->inbox, 0, 3 * h->comp * 4));  // the pitch padding stays zero
            CK(h, cudaStreamCreateWithFlags(&h->xfer, cudaStreamNonBlocking));
            CK(h, cudaEventCreateWithFlags(&h->in_ready, cudaEventDisableTiming));
            CK(h, cudaEventCreateWithFlags(&h->inbox_free, cudaEventDisableTiming));
            CK(h, cudaEventRecord(h->inbox_free, h->stream));
        }
        CK(h, cudaStreamWaitEvent(h->xfer, h->inbox_free, 0));  // the previous move out of the inbox
        for (int a = 0; a < 3; ++a) {
            int rc = put_component(h, (char*)h->inbox + (size_t)a * h->comp * 4, src[a], a, h->xfer);
            if (rc) return rc;
        }
        CK(h, cudaEventRecord(h->in_ready, h->xfer));
        CK(h, cudaStreamWaitEvent(h->stream, h->in_ready, 0));
        CK(h, cudaMemcpyAsync(h->state_base[h->cur], h->inbox, 3 * h->comp * 4, cudaMemcpyDeviceToDevice, h->stream));
        CK(h, cudaEventRecord(h->inbox_free, h->stream));
    } else {
        for (int b = 0; b < h->nb; ++b)
            for (int a = 0; a < 3; ++a) {
                void* dst = (char*)h->state[h->cur][a] + (size_t)b * 3 * h->comp * h->esz;
                int rc = put_component(h, dst, src[a] + (size_t)b * h->nvox, (3 * b + a) % h->nstage, h->stream);
                if (rc) return rc;
            }
    }
    // FP32: the host arrays have been read (converted into the staging
    // slots); the copies and the frame change complete in the handle's
    // stream order. FP64 copies read the caller's arrays directly, so they
    // finish before the call returns.
    int rc = frame_change(h, h->state[h->cur], +1);
    if (rc) return rc;
    if (h->esz == 8) CK(h, cudaStreamSynchronize(h->stream));
    return BT_OK;
}

int bt_set_state_device(bt_handle* h, const void* mx, const void* my, const void* mz) {
    if (!h || !mx || !my || !mz) return fail(h, BT_E_ARG, "null field");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    const bt_config& c = h->cfg;
    const void* src[3] = {mx, my, mz};
    for (int b = 0; b < h->nb; ++b)
        for (int a = 0; a < 3; ++a)
            CK(h, cudaMemcpy2DAsync((char*)h->state[h->cur][a] + (size_t)b * 3 * h->comp * h->esz, h->pitch * h->esz,
                                    (const char*)src[a] + (size_t)b * h->nvox * h->esz, c.nx * h->esz, c.nx * h->esz,
                                    (size_t)c.ny * c.nz, cudaMemcpyDeviceToDevice, h->stream));
    return frame_change(h, h->state[h->cur], +1);
}

int bt_get_state(bt_handle* h, double* mx, double* my, double* mz) {
    if (!h || !mx || !my || !mz) return fail(h, BT_E_ARG, "null field");
    const bool phase = any_phase(h);
    // the idle ping-pong buffer holds the lab-frame copy; the next step overwrites it
    void** src = h->state[h->cur];
    void** tmp = h->state[1 - h->cur];
    if (phase) {
        CK(h, cudaMemcpyAsync(h->state_base[1 - h->cur], h->state_base[h->cur], 3 * h->nb * h->esz * h->comp,
                              cudaMemcpyDeviceToDevice, h->stream));
        int rc = frame_change(h, tmp, -1);
        if (rc) return rc;
    }
    double* dst[3] = {mx, my, mz};
    void** from = phase ? tmp : src;
    std::vector<double*> to;
    std::vector<const void*> fr;
    for (int b = 0; b < h->nb; ++b)
        for (int a = 0; a < 3; ++a) {
            to.push_back(dst[a] + (size_t)b * h->nvox);
            fr.push_back((const char*)from[a] + (size_t)b * 3 * h->comp * h->esz);
        }
    return get_components(h, to.data(), fr.data(), (int)to.size());
}

int bt_set_schedule(bt_handle* h, const bt_pulse* pulses, int npulses, const double* grad_wave, long long nwave) {
    if (!h || npulses < 0 || (npulses > 0 && !pulses) || nwave < 0 || (nwave > 0 && !grad_wave))
        return fail(h, BT_E_ARG, "bad schedule arguments");
    CK(h, cudaStreamSynchronize(h->stream));
    return build_schedule(h, pulses, npulses, grad_wave, nwave);
}

long long bt_step_index(const bt_handle* h) { return h ? h->step : -1; }

int bt_set_step(bt_handle* h, long long step) {
    if (!h || step < 0) return fail(h, BT_E_ARG, "bad step");
    CK(h, cudaStreamSynchronize(h->stream));
    h->step = step;
    h->ctl_h->step = step;
    h->ctl_h->mt_base = step;
    h->ctl_h->ticket = 0;
    h->ctl_h->status = 0;
    CK(h, cudaMemcpy(h->ctl_d, h->ctl_h, sizeof(bt::Ctl), cudaMemcpyHostToDevice));
    return BT_OK;
}

// checks and device control block for a run of nsteps from the current step
int run_begin(bt_handle* h, long long nsteps) {
    if (!h || nsteps < 0) return fail(h, BT_E_ARG, "bad step count");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    const bt_config& c = h->cfg;
    if (c.scheme == BT_SCHEME_KSPACE && (c.grad[0] != 0.0 || c.grad[1] != 0.0 || c.grad[2] != 0.0) &&
        h->step + nsteps > h->nsched)
        return fail(h, BT_E_ARG, "KSPACE with a gradient needs a waveform covering every step run");
    int rc = ensure_mt(h, nsteps);
    if (rc) return rc;
    // ctl: step and mt_base for this run (written in stream order)
    CK(h, cudaStreamSynchronize(h->stream));
    h->ctl_h->step = h->step;
    h->ctl_h->mt_base = h->step;
    h->ctl_h->ticket = 0;
    h->ctl_h->status = 0;
    CK(h, cudaMemcpyAsync(h->ctl_d, h->ctl_h, sizeof(bt::Ctl), cudaMemcpyHostToDevice, h->stream));
    h->fast_pending = false;  // a run that failed part-way may have left one
    h->last_run = nsteps;
    return BT_OK;
}

// enqueue steps [*s, min(end, *s + limit)) on the handle's stream: runs of
// GRAPH_STEPS pulse-free steps from a graph captured once per input side,
// single launches otherwise
int run_advance(bt_handle* h, long long* s, long long end, long long limit) {
    const long long stop = std::min(end, *s + limit);
    while (*s < stop) {
        bool clean = stop - *s >= GRAPH_STEPS;
        for (long long q = *s; clean && q < *s + GRAPH_STEPS; ++q) clean = !step_has_pulse(h, q);
        if (clean) {
            // a graph starts and ends with no fast step pending
            CK(h, finish_fast(h));
            cudaGraphExec_t& g = h->graph[h->cur];
            if (!g) {
                cudaGraph_t graph;
                CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = cudaSuccess;
                const long long before = h->launches;
                for (int q = 0; q < GRAPH_STEPS && e == cudaSuccess; ++q) e = launch_one(h, (h->cur + q) & 1, *s + q);
                if (e == cudaSuccess) e = finish_fast(h);
                h->fast_pending = false;
                h->graph_launches[h->cur] = h->launches - before;
                h->launches = before;
                cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
                CK(h, e);
                CK(h, e2);
                e = cudaGraphInstantiate(&g, graph, 0);
                cudaGraphDestroy(graph);
                CK(h, e);
            }
            CK(h, cudaGraphLaunch(g, h->stream));
            h->launches += h->graph_launches[h->cur];
            *s += GRAPH_STEPS;
        } else {
            CK(h, launch_one(h, h->cur, *s));
            h->cur ^= 1;
            *s += 1;
        }
    }
    CK(h, finish_fast(h));
    h->step = *s;
    return BT_OK;
}

int bt_run_async(bt_handle* h, long long nsteps) {
    int rc = run_begin(h, nsteps);
    if (rc) return rc;
    long long s = h->step;
    return run_advance(h, &s, h->step + nsteps, nsteps);
}

int bt_run_many(bt_handle* const* hs, int n, long long nsteps) {
    if (!hs || n < 0 || nsteps < 0) return BT_E_ARG;
    for (int i = 0; i < n; ++i)
        if (!hs[i]) return BT_E_ARG;
    // the handles share the GPU: their fast paths get z-chunks such that all
    // of them together launch about two waves of two CTAs per SM, each
    // handle's share in proportion to its voxels (a handle alone would take
    // four waves by itself, and many short chunks pay many CTA prologues;
    // 48 samples of 48..192 voxels a side: 2 waves 0.599 of the roofline,
    // 3 waves 0.597, 4 waves 0.588, 6 waves 0.593)
    if (n > 1) {
        long long vox_all = 0;
        for (int i = 0; i < n; ++i)
            if (hs[i]->use_tma) vox_all += (long long)hs[i]->nvox * hs[i]->nb;
        for (int i = 0; i < n && vox_all > 0; ++i) {
            bt_handle* h = hs[i];
            if (!h->use_tma) continue;
            const bt_config& c = h->cfg;
            const int tw = h->ttx, th = bt::tile_rows(tw);
            const double tiles = (double)((c.nx + tw - 1) / tw) * ((c.ny + th - 1) / th);
            // this handle's share of the CTAs, per member, as a chunk count
            const double want = 4.0 * h->num_sms * ((double)h->nvox / (double)vox_all);
            const long long ch = (long long)std::max(tiles, std::min(std::floor(want + 0.5), tiles * std::max(1, c.nz / 8)));
            if (ch != (long long)(h->tzsplit - 1) * tma_tiles(h) + h->tzlong) {
                CK(h, cudaStreamSynchronize(h->stream));
                int rc = set_tma_chunks(h, ch);
                if (rc) return rc;
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        int rc = run_begin(hs[i], nsteps);
        if (rc) return rc;
    }
    std::vector<long long> pos(n), end(n);
    for (int i = 0; i < n; ++i) {
        pos[i] = hs[i]->step;
        end[i] = hs[i]->step + nsteps;
    }
    // round robin, one graph's worth of steps per handle per round, so that
    // handles whose streams share a hardware queue still interleave
    for (bool more = true; more;) {
        more = false;
        for (int i = 0; i < n; ++i) {
            if (pos[i] >= end[i]) continue;
            int rc = run_advance(hs[i], &pos[i], end[i], GRAPH_STEPS);
            if (rc) return rc;
            more = more || pos[i] < end[i];
        }
    }
    return BT_OK;
}

int bt_read_mt(bt_handle* h, double* mt_out, long long nsteps) {
    if (!h || nsteps < 0 || nsteps > h->last_run) return fail(h, BT_E_ARG, "bad M(t) read");
    int rc = check_ctl(h);
    if (rc) return rc;
    if (mt_out && nsteps > 0)
        CK(h, cudaMemcpy(mt_out, h->mt_d, sizeof(double) * 3 * nsteps * h->nb, cudaMemcpyDeviceToHost));
    return BT_OK;
}

int bt_run(bt_handle* h, long long nsteps, double* mt_out) {
    int rc = bt_run_async(h, nsteps);
    if (rc) return rc;
    return bt_read_mt(h, mt_out, nsteps);
}

int bt_synchronize(bt_handle* h) {
    if (!h) return BT_E_ARG;
    CK(h, cudaStreamSynchronize(h->stream));
    return BT_OK;
}

void* bt_stream(bt_handle* h) { return h ? (void*)h->stream : nullptr; }

int bt_measure(bt_handle* h, double* sums3) {
    if (!h || !sums3) return fail(h, BT_E_ARG, "null output");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    std::vector<double> part(4 * SUMS_BLOCKS);
    for (int b = 0; b < h->nb; ++b) {
        double kv[4];
        kvec_at(h, h->step, b, kv);
        kv[3] = SUMS_BLOCKS;
        cudaError_t e;
        if (h->esz == 8) {
            bt::StepParams<double> P = h->pd[h->cur];
            for (int a = 0; a < 3; ++a) P.in[a] += (size_t)b * 3 * h->comp;
            e = bt::launch_sums<double>(P, kv, h->stream);
        } else {
            bt::StepParams<float> P = h->pf[h->cur];
            for (int a = 0; a < 3; ++a) P.in[a] += (size_t)b * 3 * h->comp;
            e = bt::launch_sums<float>(P, kv, h->stream);
        }
        CK(h, e);
        h->launches++;
        CK(h, cudaMemcpyAsync(part.data(), h->partials_d, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                              h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        double t[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < SUMS_BLOCKS; ++q)
            for (int a = 0; a < 3; ++a) t[a] += part[4 * q + a];
        for (int a = 0; a < 3; ++a) sums3[3 * b + a] = t[a];
    }
    return BT_OK;
}

long long bt_launch_count(const bt_handle* h) { return h ? h->launches : -1; }

namespace {

// dense [nz][ny][nx] doubles -> count pitched arrays of the handle's precision
int put_pitched(bt_handle* h, void* dst, const std::vector<double>& src, int count) {
    const bt_config& c = h->cfg;
    CK(h, cudaStreamSynchronize(h->stream));
    const size_t n = (size_t)count * h->comp;
    if (h->esz == 8) {
        CK(h, cudaMemcpy(dst, src.data(), n * 8, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> f(n);
        convert(f.data(), src.data(), n);
        CK(h, cudaMemcpy(dst, f.data(), n * 4, cudaMemcpyHostToDevice));
    }
    (void)c;
    return BT_OK;
}

// Open-addressing table of at most 512 rate pairs (1024 slots): each key's
// insertion index. The palette build looks up every pore voxel's pair.
struct PairTable {
    uint64_t key[1024];
    int16_t val[1024];  // insertion index, -1 = empty slot
    int n = 0;
    PairTable() { std::fill(val, val + 1024, (int16_t)-1); }
    static unsigned slot(uint64_t k) {
        k ^= k >> 33;
        k *= 0xff51afd7ed558ccdULL;
        k ^= k >> 33;
        return (unsigned)k & 1023u;
    }
    // the key's index, inserted as the next one if new; -1 if new and the
    // table already holds cap keys
    int find_or_add(uint64_t k, int cap) {
        for (unsigned s = slot(k);; s = (s + 1) & 1023u) {
            if (val[s] < 0) {
                if (n >= cap) return -1;
                key[s] = k;
                val[s] = (int16_t)n;
                return n++;
            }
            if (key[s] == k) return val[s];
        }
    }
    int find(uint64_t k) const {
        for (unsigned s = slot(k);; s = (s + 1) & 1023u) {
            if (val[s] < 0) return -1;
            if (key[s] == k) return val[s];
        }
    }
};

// FP32 handles take per-voxel rates through a rate palette when they fit
// one: the pore voxels' diffusivity is the configuration's (so the code
// table's face weights hold), the solid voxels' is negligible (at most 1e-20
// m^2/s: its face weights vanish in FP32 either way), and the pore voxels'
// FP32 (dTime*(1/T1), dTime*(1/T2)) pairs take at most 256 values. Then each
// voxel gets its pair's index (solid voxels index 0: their update is zero),
// and the fast path and the generic kernel read the pair from the palette;
// otherwise the generic kernel reads the eight per-voxel fields.
int build_palette(bt_handle* h, const double* t1, const double* t2, const double* diff) {
    const bt_config& c = h->cfg;
    h->pal_ok = false;
    if (c.precision != BT_F32 || c.scheme == BT_SCHEME_MACCORMACK || h->mask_h.size() != h->nvox) return BT_OK;
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const double dTime = c.dt;
    // the FP32 pair of voxel q, formed as the per-voxel fields form it
    auto key_at = [&](size_t q) {
        const float r1 = (float)(dTime * (1.0 / t1[q])), r2 = (float)(dTime * (1.0 / t2[q]));
        uint32_t b1, b2;
        std::memcpy(&b1, &r1, 4);
        std::memcpy(&b2, &r2, 4);
        return ((uint64_t)b1 << 32) | b2;
    };
    // pass 1, planes in parallel: each slice's distinct pairs in first-seen
    // order (at most 257 kept: one more means no palette) and the diffusivity
    // checks
    const size_t grain = std::max<size_t>(1, ((size_t)1 << 18) / ((size_t)nx * ny));
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nsl = std::max<size_t>(1, std::min<size_t>(std::min(hw, 32u), (size_t)nz / grain));
    std::vector<std::vector<uint64_t>> found(nsl);
    std::vector<char> bad(nsl, 0);
    parallel_slices(nsl, 1, [&](size_t sa, size_t sb) {
        std::unique_ptr<PairTable> seen(new PairTable);
        for (size_t sl = sa; sl < sb; ++sl) {
            std::vector<uint64_t>& mine = found[sl];
            *seen = PairTable();
            uint64_t last = ~0ull;
            for (int k = (int)(nz * sl / nsl); k < (int)(nz * (sl + 1) / nsl) && !bad[sl]; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        const size_t q = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                        if (!h->mask_h[q]) {
                            if (!(diff[q] <= 1e-20)) bad[sl] = 1;
                            continue;
                        }
                        if (diff[q] != c.d_pore) bad[sl] = 1;
                        const uint64_t key = key_at(q);
                        if (key == last) continue;
                        last = key;
                        const int before = seen->n;
                        const int at = seen->find_or_add(key, 257);
                        if (at < 0) {
                            bad[sl] = 1;
                            break;
                        }
                        if (at == before) mine.push_back(key);
                    }
        }
    });
    // the palette: the slices' pairs in slice order, then first-seen order
    std::unique_ptr<PairTable> id(new PairTable);
    std::vector<float> tab(512, 0.f);
    for (size_t sl = 0; sl < nsl; ++sl) {
        if (bad[sl]) return BT_OK;
        for (uint64_t key : found[sl]) {
            const int before = id->n;
            const int n = id->find_or_add(key, 256);
            if (n < 0) return BT_OK;
            if (n == before) {
                const uint32_t b1 = (uint32_t)(key >> 32), b2 = (uint32_t)key;
                std::memcpy(&tab[2 * n], &b1, 4);
                std::memcpy(&tab[2 * n + 1], &b2, 4);
            }
        }
    }
    // pass 2, planes in parallel: each voxel's index (solid voxels 0)
    std::vector<uint8_t> idx((size_t)nz * ny * h->cpitch, 0);
    parallel_slices((size_t)nz, grain, [&](size_t ka, size_t kb) {
        uint64_t last = ~0ull;
        int last_id = 0;
        for (int k = (int)ka; k < (int)kb; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const size_t q = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                    if (!h->mask_h[q]) continue;
                    const uint64_t key = key_at(q);
                    if (key != last) {
                        last = key;
                        last_id = id->find(key);
                    }
                    idx[((size_t)k * ny + j) * h->cpitch + i] = (uint8_t)last_id;
                }
    });
    CK(h, cudaStreamSynchronize(h->stream));
    if (!h->pal_idx) CK(h, cudaMalloc(&h->pal_idx, idx.size()));
    if (!h->pal_tab) CK(h, cudaMalloc(&h->pal_tab, 512 * sizeof(float)));
    CK(h, cudaMemcpy(h->pal_idx, idx.data(), idx.size(), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->pal_tab, tab.data(), 512 * sizeof(float), cudaMemcpyHostToDevice));
    // the tensor maps gain the palette index
    if (h->use_tma) h->use_tma = build_maps(h);
    h->pal_ok = true;
    return BT_OK;
}

}  // namespace

int bt_upload_rates(bt_handle* h, const double* t1, const double* t2, const double* diff) {
    if (!h) return BT_E_ARG;
    if (!t1 && !t2 && !diff) {
        CK(h, cudaStreamSynchronize(h->stream));
        if (h->fields_d) cudaFree(h->fields_d);
        h->fields_d = nullptr;
        h->pal_ok = false;
        refresh_params(h);
        return BT_OK;
    }
    if (!t1 || !t2 || !diff) return fail(h, BT_E_ARG, "t1, t2 and diff are uploaded together");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    // rates that fit the rate palette need no per-voxel fields
    int rc = build_palette(h, t1, t2, diff);
    if (rc) return rc;
    if (h->pal_ok) {
        CK(h, cudaStreamSynchronize(h->stream));
        if (h->fields_d) cudaFree(h->fields_d);
        h->fields_d = nullptr;
        refresh_params(h);
        return BT_OK;
    }
    const bt_config& c = h->cfg;
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const size_t comp = h->comp;
    std::vector<double> buf(8 * comp, 0.0);
    const double dTime = c.dt;
    const double reg = c.scheme == BT_SCHEME_MACCORMACK ? 1.0e-25 : SMALL;
    // planes in parallel on the host's cores
    parallel_slices((size_t)nz, std::max<size_t>(1, ((size_t)1 << 18) / ((size_t)nx * ny)), [&](size_t ka, size_t kb) {
    for (int k = (int)ka; k < (int)kb; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t q = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                const size_t v = ((size_t)k * ny + j) * h->pitch + i;
                // ExplicitSimple (cpp:3174-3185): tau = 1/relTime, relaxation dTime*tau
                buf[v] = dTime * (1.0 / t1[q]);
                buf[comp + v] = dTime * (1.0 / t2[q]);
                // harmonic-mean face diffusivities; ghosts copy the edge value
                // (BoundaryConditionsForDiffusion), so a domain face pairs the voxel with itself
                const double Dc = diff[q];
                const double nb[6] = {i > 0 ? diff[q - 1] : Dc, i < nx - 1 ? diff[q + 1] : Dc,
                                      j > 0 ? diff[q - nx] : Dc, j < ny - 1 ? diff[q + nx] : Dc,
                                      k > 0 ? diff[q - (size_t)nx * ny] : Dc,
                                      k < nz - 1 ? diff[q + (size_t)nx * ny] : Dc};
                for (int f = 0; f < 6; ++f) buf[(2 + f) * comp + v] = 2.0 * (nb[f] * Dc) / (nb[f] + Dc + reg);
            }
    });
    if (!h->fields_d) {
        drop_graphs(h);
        CK(h, cudaMalloc(&h->fields_d, 8 * comp * h->esz));
    }
    rc = put_pitched(h, h->fields_d, buf, 8);
    if (rc) return rc;
    refresh_params(h);
    return BT_OK;
}

int bt_upload_rate_palette(bt_handle* h, const double* t1, const double* t2, int n, const void* idx) {
    if (!h) return BT_E_ARG;
    const bt_config& c = h->cfg;
    if (!t1 || !t2 || !idx || n < 1 || n > 256) return fail(h, BT_E_ARG, "a palette of 1..256 entries and its index");
    if (c.precision != BT_F32 || c.scheme == BT_SCHEME_MACCORMACK)
        return fail(h, BT_E_ARG, "rate palettes are for FP32 handles outside the MacCormack scheme");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    // each entry's FP32 pair, formed as the per-voxel fields form it
    std::vector<float> tab(512, 0.f);
    for (int e = 0; e < n; ++e) {
        tab[2 * e] = (float)(c.dt * (1.0 / t1[e]));
        tab[2 * e + 1] = (float)(c.dt * (1.0 / t2[e]));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->fields_d) cudaFree(h->fields_d);
    h->fields_d = nullptr;
    if (!h->pal_idx) CK(h, cudaMalloc(&h->pal_idx, (size_t)c.nz * c.ny * h->cpitch));
    if (!h->pal_tab) CK(h, cudaMalloc(&h->pal_tab, 512 * sizeof(float)));
    CK(h, cudaMemcpy2DAsync(h->pal_idx, h->cpitch, idx, c.nx, c.nx, (size_t)c.ny * c.nz, cudaMemcpyDeviceToDevice,
                            h->stream));
    CK(h, cudaMemcpyAsync(h->pal_tab, tab.data(), 512 * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));  // tab is a host temporary
    if (h->use_tma) h->use_tma = build_maps(h);
    h->pal_ok = true;
    refresh_params(h);
    return BT_OK;
}

int bt_set_phase_weights(bt_handle* h, const double* c1, const double* c2) {
    if (!h) return BT_E_ARG;
    if (!c1 && !c2) {
        CK(h, cudaStreamSynchronize(h->stream));
        drop_graphs(h);
        if (h->weights_d) cudaFree(h->weights_d);
        if (h->part6_d) cudaFree(h->part6_d);
        h->weights_d = nullptr;
        h->part6_d = nullptr;
        return BT_OK;
    }
    if (!c1 || !c2) return fail(h, BT_E_ARG, "c1 and c2 are set together");
    if (h->nb > 1) return fail(h, BT_E_ARG, "two-component sums take one field per handle");
    if (h->cfg.scheme == BT_SCHEME_KSPACE) return fail(h, BT_E_ARG, "two-component sums are lab-frame sums: not KSPACE");
    if (!h->geometry || !h->mask_h.size()) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    const bt_config& c = h->cfg;
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const size_t comp = h->comp;
    std::vector<double> buf(2 * comp, 0.0);
    const int x0 = c.buffer[0], x1 = nx - c.buffer[0], y0 = c.buffer[1], y1 = ny - c.buffer[1];
    const int z0 = c.buffer[2], z1 = nz - c.buffer[2];
    for (int k = z0; k < z1; ++k)
        for (int j = y0; j < y1; ++j)
            for (int i = x0; i < x1; ++i) {
                const size_t q = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                // OutputX/Y/Z (cpp:3324-3350): pore voxels where one phase exceeds 0.8
                if (!h->mask_h[q] || !(c1[q] > 0.8 || c2[q] > 0.8)) continue;
                const size_t v = ((size_t)k * ny + j) * h->pitch + i;
                buf[v] = c1[q];
                buf[comp + v] = c2[q];
            }
    if (!h->weights_d) {
        CK(h, cudaStreamSynchronize(h->stream));
        drop_graphs(h);
        CK(h, cudaMalloc(&h->weights_d, 2 * comp * h->esz));
        CK(h, cudaMalloc(&h->part6_d, sizeof(double) * 6 * SUMS_BLOCKS));
    }
    return put_pitched(h, h->weights_d, buf, 2);
}

int bt_read_mt_phases(bt_handle* h, double* out, long long nsteps) {
    if (!h || !out || nsteps < 0 || nsteps > h->last_run) return fail(h, BT_E_ARG, "bad two-component M(t) read");
    if (!h->weights_d) return fail(h, BT_E_STATE, "bt_set_phase_weights first");
    int rc = check_ctl(h);
    if (rc) return rc;
    if (nsteps > 0) CK(h, cudaMemcpy(out, h->mt6_d, sizeof(double) * 6 * nsteps, cudaMemcpyDeviceToHost));
    return BT_OK;
}

int bt_field_device(bt_handle* h, int member, void** mx, void** my, void** mz, int* pitch) {
    if (!h || member < 0 || member >= h->nb || !mx || !my || !mz || !pitch) return fail(h, BT_E_ARG, "bad field query");
    const size_t off = (size_t)member * 3 * h->comp * h->esz;
    *mx = (char*)h->state[h->cur][0] + off;
    *my = (char*)h->state[h->cur][1] + off;
    *mz = (char*)h->state[h->cur][2] + off;
    *pitch = h->pitch;
    return BT_OK;
}

int bt_set_wait_polls(bt_handle* h, long long polls) {
    if (!h) return BT_E_ARG;
    CK(h, cudaStreamSynchronize(h->stream));
    h->wait_polls = polls < 0 ? bt::RING_WAIT_POLLS : (uint32_t)std::min<long long>(polls, 0xffffffffLL);
    refresh_params(h);  // the parameters are baked into the captured graphs
    return BT_OK;
}

int bt_set_tma_split(bt_handle* h, int zsplit) {
    if (!h) return BT_E_ARG;
    if (h->cfg.precision != BT_F32 || !h->use_tma) return BT_OK;  // no fast path on this handle
    CK(h, cudaStreamSynchronize(h->stream));
    return set_tma_split(h, zsplit > 0 ? zsplit : default_tma_split(h));
}

int bt_set_tma_chunks(bt_handle* h, int chunks) {
    if (!h) return BT_E_ARG;
    if (h->cfg.precision != BT_F32 || !h->use_tma) return BT_OK;  // no fast path on this handle
    CK(h, cudaStreamSynchronize(h->stream));
    if (chunks <= 0) return set_tma_split(h, default_tma_split(h));
    return set_tma_chunks(h, chunks);
}

int bt_autotune(bt_handle* h, int trial_steps, int* best_chunks) {
    if (!h || trial_steps <= 0) return fail(h, BT_E_ARG, "bad autotune arguments");
    if (!h->geometry) return fail(h, BT_E_STATE, "bt_upload_geometry first");
    if (h->cfg.precision != BT_F32 || !h->use_tma) {
        if (best_chunks) *best_chunks = h->gzsplit;
        return BT_OK;
    }
    // candidate chunkings (chunks per field): for 1 to 8 waves of 2 CTAs per
    // SM, and for the first four wave counts at which every tile column has a
    // chunk (a batch's members share the waves), the chunk count that fills
    // exactly that many waves (tile columns differing by one chunk) and the
    // even splits just below and just above it; chunks of >= 4 planes
    const bt_config& c = h->cfg;
    const long long tiles = tma_tiles(h);
    const long long slots_all = 2LL * h->num_sms;  // CTA slots of the GPU
    std::vector<long long> cand;
    auto add = [&](long long chunks) {
        if (chunks >= tiles && chunks <= tiles * std::max(1, c.nz / 4)) cand.push_back(chunks);
    };
    const long long w_min = (tiles * h->nb + slots_all - 1) / slots_all;  // waves with one chunk per column
    for (long long waves = 1; waves <= std::max<long long>(8, w_min + 3); ++waves) {
        if (waves > 8 && waves < w_min) continue;
        const long long fill = waves * slots_all / h->nb;  // chunks per member
        const long long below = fill / tiles;
        add(fill);
        add(below * tiles);
        add((below + 1) * tiles);
    }
    cand.push_back((long long)default_tma_split(h) * tiles);
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    // the trial runs advance the field; the caller's field and step are restored
    const long long step0 = h->step;
    const int cur0 = h->cur;
    void* keep = nullptr;
    const size_t sbytes = 3 * h->esz * h->comp * h->nb;
    CK(h, cudaMalloc(&keep, sbytes));
    CK(h, cudaMemcpyAsync(keep, h->state_base[h->cur], sbytes, cudaMemcpyDeviceToDevice, h->stream));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    long long best_ch = (long long)(h->tzsplit - 1) * tiles + h->tzlong;
    int rc = BT_OK;
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    for (long long ch : cand) {
        if ((rc = set_tma_chunks(h, ch))) break;
        if ((rc = bt_run_async(h, GRAPH_STEPS))) break;  // warm-up and graph capture
        cudaEventRecord(e0, h->stream);
        if ((rc = bt_run_async(h, trial_steps))) break;
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if ((rc = check_ctl(h))) break;
        if (ms < best) {
            best = ms;
            best_ch = ch;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(h->stream);
    h->cur = cur0;
    cudaMemcpy(h->state_base[h->cur], keep, sbytes, cudaMemcpyDeviceToDevice);
    cudaFree(keep);
    if (rc) return rc;
    rc = set_tma_chunks(h, best_ch);
    if (rc) return rc;
    rc = bt_set_step(h, step0);
    if (rc) return rc;
    if (best_chunks) *best_chunks = (int)((long long)(h->tzsplit - 1) * tiles + h->tzlong);
    return BT_OK;
}

}  // extern "C"
