// Harness for the reference solver's own CUDA kernels — TEST INFRASTRUCTURE ONLY.
//
// The reference's kernels (NMR_predictor_upgrade, NMR_corrector_upgrade and
// the BC_* ghost-layer kernels of src/NmrRelaxationSolveKernels.cu) are
// compiled unmodified from the reference sources into a cubin by
// oracle/Makefile (target ref-gpu); this file loads that cubin through the
// CUDA driver API and drives the kernels the way the reference's host code
// does, restated here:
//   InitializeGpu (cu:12-88): FP64 ghosted arrays on the device, copied as
//       given (the caller builds them; oracle bto_gpu_inputs restates the
//       reference's set-up), predictor and corrector arrays zeroed;
//   solve_gpu's loop (cu:1187-1288), per step: ExplicitMakUpgrade; pulses
//       (Sequence_gpu) are not applied here; BoundaryConditionsForVectorField_gpu
//       on the field; every ndprint steps the three full-field device-to-host
//       copies and OutputX/Y/Z (cpp:3301-3461, one component);
//   ExplicitMakUpgrade (cu:1473-1501): predictor (grid ceil(ik*jk/128) x kk,
//       128 threads), ghost layers of the predictor, corrector, ghost layers of
//       the corrector, three device-to-device copies corrector -> field;
//   BoundaryConditionsForVectorField_gpu (cu:1321-1396): the BC kernel
//       dispatch on nBoundary1..6 with 32 x 32 blocks.
// Everything runs on the context's legacy default stream, as the reference.
// The reference's unused device arrays (addMagnetization, softner) are not
// allocated. Kernel handles are found by enumerating the module's functions.
#include <cuda.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace {

// include_lib.h:23, passed by value to every kernel
struct GridSize {
    int ik, jk, kk, num;
};

struct Module {
    CUmodule mod = nullptr;
    CUfunction pred = nullptr, corr = nullptr;
    CUfunction zero_der[3] = {}, inf[3] = {}, adv_xm = nullptr, adv_xp = nullptr;
};

thread_local std::string g_err;
std::mutex g_mutex;
// modules per (context, cubin path); the primary contexts the harness uses
// are retained once and kept for the life of the process, so a module never
// outlives its context (releasing the last reference would destroy the
// context and every module loaded in it)
std::map<std::pair<CUcontext, std::string>, Module> g_modules;
std::map<CUdevice, CUcontext> g_contexts;

bool ck(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "unknown CUDA driver error");
    return false;
}

// the kernel whose Itanium-mangled name is _Z<len><name><parameters>
CUfunction find(CUmodule mod, const char* name) {
    unsigned n = 0;
    if (cuModuleGetFunctionCount(&n, mod) != CUDA_SUCCESS || n == 0) return nullptr;
    std::vector<CUfunction> fs(n);
    if (cuModuleEnumerateFunctions(fs.data(), n, mod) != CUDA_SUCCESS) return nullptr;
    const std::string want = "_Z" + std::to_string(std::strlen(name)) + name;
    for (CUfunction f : fs) {
        const char* fn = nullptr;
        if (cuFuncGetName(&fn, f) == CUDA_SUCCESS && fn && std::strncmp(fn, want.c_str(), want.size()) == 0)
            return f;
    }
    return nullptr;
}

// the device's primary context, retained on first use and never released
CUcontext primary_context(CUdevice dev) {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_contexts.find(dev);
    if (it != g_contexts.end()) return it->second;
    CUcontext c = nullptr;
    if (!ck(cuDevicePrimaryCtxRetain(&c, dev), "cuDevicePrimaryCtxRetain")) return nullptr;
    g_contexts[dev] = c;
    return c;
}

// with the module's context current
Module* load(CUcontext ctx, const char* path) {
    std::lock_guard<std::mutex> lock(g_mutex);
    const auto key = std::make_pair(ctx, std::string(path));
    auto it = g_modules.find(key);
    if (it != g_modules.end()) return &it->second;
    Module m;
    if (!ck(cuModuleLoad(&m.mod, path), "cuModuleLoad")) return nullptr;
    m.pred = find(m.mod, "NMR_predictor_upgrade");
    m.corr = find(m.mod, "NMR_corrector_upgrade");
    const char* zd[3] = {"BC_ZeroDer_X", "BC_ZeroDer_Y", "BC_ZeroDer_Z"};
    const char* in[3] = {"BC_Inf_X", "BC_Inf_Y", "BC_Inf_Z"};
    for (int a = 0; a < 3; ++a) {
        m.zero_der[a] = find(m.mod, zd[a]);
        m.inf[a] = find(m.mod, in[a]);
        if (!m.zero_der[a] || !m.inf[a]) {
            g_err = "reference BC kernel not found in the cubin";
            return nullptr;
        }
    }
    m.adv_xm = find(m.mod, "BC_Advanced_XM");
    m.adv_xp = find(m.mod, "BC_Advanced_XP");
    if (!m.pred || !m.corr || !m.adv_xm || !m.adv_xp) {
        g_err = "reference kernel not found in the cubin";
        return nullptr;
    }
    // InitializeGpu's cudaDeviceSetCacheConfig(cudaFuncCachePreferL1), per kernel
    CUfunction all[] = {m.pred, m.corr};
    for (CUfunction f : all) cuFuncSetCacheConfig(f, CU_FUNC_CACHE_PREFER_L1);
    return &g_modules.emplace(key, m).first->second;
}

// RAII: the device's primary context current for the duration of a call
struct CtxScope {
    bool ok = false;
    CtxScope(CUcontext c) { ok = ck(cuCtxPushCurrent(c), "cuCtxPushCurrent"); }
    ~CtxScope() {
        CUcontext c;
        if (ok) cuCtxPopCurrent(&c);
    }
};

}  // namespace

extern "C" {

typedef struct rg_params {
    int ik, jk, kk;          // interior cells
    double dt, dx, dy, dz;
    int vector_mult, velocity, diffusion;
    double p_eq;
    int nb[6];               // nBoundary1..6 (x-: 1, y-: 2, x+: 3, y+: 4, z-: 5, z+: 6)
    int buffer[3];           // bufferSizeX/Y/Z of OutputX/Y/Z
} rg_params;

struct rg_handle {
    Module* m = nullptr;
    CUcontext ctx = nullptr;
    CUdevice dev = 0;
    rg_params p{};
    GridSize gs{};
    size_t num = 0;
    CUdeviceptr act = 0, diff = 0, t1 = 0, t2 = 0;
    CUdeviceptr mag[3] = {}, mf[3] = {}, nf[3] = {}, vel[3] = {}, pr[3] = {}, co[3] = {};
    std::vector<char> act_h;
    std::vector<double> host[3];
};

const char* rg_last_error(void) { return g_err.c_str(); }

void rg_destroy(rg_handle* h) {
    if (!h) return;
    if (h->ctx) {
        CtxScope s(h->ctx);
        CUdeviceptr* ptrs[] = {&h->act, &h->diff, &h->t1, &h->t2};
        for (auto* q : ptrs)
            if (*q) cuMemFree(*q);
        for (int a = 0; a < 3; ++a) {
            CUdeviceptr q3[] = {h->mag[a], h->mf[a], h->nf[a], h->vel[a], h->pr[a], h->co[a]};
            for (CUdeviceptr q : q3)
                if (q) cuMemFree(q);
        }
    }
    delete h;
}

// arrays: ghosted (ik+2)(jk+2)(kk+2) cells, x fastest; mf, nf, vel, magn hold
// the x, y, z components one after another (3*num)
rg_handle* rg_create(const char* cubin, int device, const rg_params* p, const char* act, const double* diff,
                     const double* t1, const double* t2, const double* mf, const double* nf, const double* vel,
                     const double* magn) {
    if (!cubin || !p || p->ik <= 0 || p->jk <= 0 || p->kk <= 0) {
        g_err = "bad arguments";
        return nullptr;
    }
    if (!ck(cuInit(0), "cuInit")) return nullptr;
    rg_handle* h = new rg_handle();
    h->p = *p;
    if (!ck(cuDeviceGet(&h->dev, device), "cuDeviceGet") || !(h->ctx = primary_context(h->dev))) {
        h->ctx = nullptr;
        rg_destroy(h);
        return nullptr;
    }
    CtxScope scope(h->ctx);
    h->m = scope.ok ? load(h->ctx, cubin) : nullptr;
    if (!scope.ok || !h->m) {
        rg_destroy(h);
        return nullptr;
    }
    h->gs = GridSize{p->ik, p->jk, p->kk, (p->ik + 2) * (p->jk + 2) * (p->kk + 2)};
    h->num = (size_t)(p->ik + 2) * (p->jk + 2) * (p->kk + 2);
    const size_t nb = h->num * sizeof(double);
    bool ok = ck(cuMemAlloc(&h->act, h->num), "cuMemAlloc") && ck(cuMemAlloc(&h->diff, nb), "cuMemAlloc") &&
              ck(cuMemAlloc(&h->t1, nb), "cuMemAlloc") && ck(cuMemAlloc(&h->t2, nb), "cuMemAlloc");
    for (int a = 0; a < 3 && ok; ++a) {
        CUdeviceptr* q3[] = {&h->mag[a], &h->mf[a], &h->nf[a], &h->vel[a], &h->pr[a], &h->co[a]};
        for (CUdeviceptr* q : q3) ok = ok && ck(cuMemAlloc(q, nb), "cuMemAlloc");
    }
    ok = ok && ck(cuMemcpyHtoD(h->act, act, h->num), "H2D") && ck(cuMemcpyHtoD(h->diff, diff, nb), "H2D") &&
         ck(cuMemcpyHtoD(h->t1, t1, nb), "H2D") && ck(cuMemcpyHtoD(h->t2, t2, nb), "H2D");
    for (int a = 0; a < 3 && ok; ++a) {
        ok = ck(cuMemcpyHtoD(h->mag[a], magn + a * h->num, nb), "H2D") &&
             ck(cuMemcpyHtoD(h->mf[a], mf + a * h->num, nb), "H2D") &&
             ck(cuMemcpyHtoD(h->nf[a], nf + a * h->num, nb), "H2D") &&
             ck(cuMemcpyHtoD(h->vel[a], vel + a * h->num, nb), "H2D") &&
             ck(cuMemsetD8(h->pr[a], 0, nb), "memset") && ck(cuMemsetD8(h->co[a], 0, nb), "memset");
    }
    if (!ok) {
        rg_destroy(h);
        return nullptr;
    }
    h->act_h.assign(act, act + h->num);
    for (auto& v : h->host) v.resize(h->num);
    return h;
}

}  // extern "C"

namespace {

bool launch(CUfunction f, unsigned gx, unsigned gy, unsigned bx, unsigned by, void** args, const char* what) {
    return ck(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, 0, nullptr, args, nullptr), what);
}

// BoundaryConditionsForVectorField_gpu (cu:1321-1396) on three device arrays
bool boundaries(rg_handle* h, CUdeviceptr* F) {
    const GridSize gs = h->gs;
    const int* nb = h->p.nb;
    const unsigned B = 32;
    const unsigned gx[2] = {(unsigned)std::ceil((double)(gs.jk + 2) / B), (unsigned)std::ceil((double)(gs.kk + 2) / B)};
    const unsigned gy[2] = {(unsigned)std::ceil((double)(gs.ik + 2) / B), (unsigned)std::ceil((double)(gs.kk + 2) / B)};
    const unsigned gz[2] = {(unsigned)std::ceil((double)(gs.ik + 2) / B), (unsigned)std::ceil((double)(gs.jk + 2) / B)};
    const unsigned* grids[3] = {gx, gy, gz};
    GridSize g = gs;
    double zero = 0.0;
    bool ok = true;
    auto each = [&](CUfunction f, const unsigned* grid, bool with_val) {
        for (int c = 0; c < 3 && ok; ++c) {
            void* a2[] = {&F[c], &g};
            void* a3[] = {&F[c], &zero, &g};
            ok = launch(f, grid[0], grid[1], B, B, with_val ? a3 : a2, "BC kernel");
        }
    };
    // pairs: x = (nBoundary1, nBoundary3), y = (2, 4), z = (5, 6)
    const int lo[3] = {nb[0], nb[1], nb[4]}, hi[3] = {nb[2], nb[3], nb[5]};
    for (int a = 0; a < 3; ++a)
        if (lo[a] == 1 && hi[a] == 1) each(h->m->zero_der[a], grids[a], false);
    for (int a = 0; a < 3; ++a)
        if (lo[a] == 3 && hi[a] == 3) each(h->m->inf[a], grids[a], false);
    if (nb[0] == 2) {
        each(h->m->adv_xm, gx, true);
        each(h->m->adv_xp, gx, true);
    }
    if (nb[2] == 2) {
        each(h->m->adv_xp, gx, true);
        each(h->m->adv_xm, gx, true);
    }
    return ok;
}

// OutputX/Y/Z (cpp:3301-3461, one component) of the host copies
void outputs(const rg_handle* h, double* out3) {
    const GridSize& gs = h->gs;
    const int bx = h->p.buffer[0], by = h->p.buffer[1], bz = h->p.buffer[2];
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = 1 + bz; k < gs.kk + 1 - bz; k++)
        for (int j = 1 + by; j < gs.jk + 1 - by; j++)
            for (int i = 1 + bx; i < gs.ik + 1 - bx; i++) {
                const size_t q = (size_t)i + (size_t)(gs.ik + 2) * ((size_t)j + (size_t)(gs.jk + 2) * k);
                if (h->act_h[q] == '1')
                    for (int c = 0; c < 3; ++c) s[c] += h->host[c][q];
            }
    for (int c = 0; c < 3; ++c) out3[c] = s[c];
}

}  // namespace

extern "C" {

// nsteps steps of solve_gpu's loop; every ndprint-th step (i % ndprint == 0)
// its three sums go to mt (3 doubles each, in order; mt may be NULL).
// *seconds: host wall time of the loop including the final synchronisation.
int rg_run(rg_handle* h, long long nsteps, long long ndprint, double* mt, double* seconds) {
    if (!h || nsteps < 0 || ndprint <= 0) {
        g_err = "bad arguments";
        return -1;
    }
    CtxScope scope(h->ctx);
    if (!scope.ok) return -2;
    rg_params& p = h->p;
    GridSize gs = h->gs;
    double dt = p.dt, dx = p.dx, dy = p.dy, dz = p.dz, peq = p.p_eq;
    int nvm = p.vector_mult, nvel = p.velocity, ndif = p.diffusion;
    void* args[] = {&h->act,   &h->diff,  &h->mag[0], &h->mag[1], &h->mag[2], &h->mf[0], &h->mf[1], &h->mf[2],
                    &h->nf[0], &h->nf[1], &h->nf[2],  &h->pr[0],  &h->pr[1],  &h->pr[2], &h->co[0], &h->co[1],
                    &h->co[2], &h->vel[0], &h->vel[1], &h->vel[2], &dt,       &dx,       &dy,       &dz,
                    &gs,       &nvm,      &nvel,      &ndif,      &h->t1,     &h->t2,    &peq};
    const unsigned g2x = (unsigned)std::ceil(gs.ik * (double)gs.jk / 128), g2y = (unsigned)gs.kk;
    const size_t nb = h->num * sizeof(double);
    long long printed = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (long long i = 0; i < nsteps; ++i) {
        // ExplicitMakUpgrade
        if (!launch(h->m->pred, g2x, g2y, 128, 1, args, "NMR_predictor_upgrade")) return -3;
        if (!boundaries(h, h->pr)) return -3;
        if (!launch(h->m->corr, g2x, g2y, 128, 1, args, "NMR_corrector_upgrade")) return -3;
        if (!boundaries(h, h->co)) return -3;
        for (int c = 0; c < 3; ++c)
            if (!ck(cuMemcpyDtoD(h->mag[c], h->co[c], nb), "D2D")) return -3;
        if (!boundaries(h, h->mag)) return -3;
        if (i % ndprint == 0) {
            for (int c = 0; c < 3; ++c)
                if (!ck(cuMemcpyDtoH(h->host[c].data(), h->mag[c], nb), "D2H")) return -3;
            if (mt) outputs(h, mt + 3 * printed);
            printed++;
        }
    }
    if (!ck(cuCtxSynchronize(), "cuCtxSynchronize")) return -3;
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

// the current field (3*num, ghosted, x y z)
int rg_get(rg_handle* h, double* magn) {
    if (!h || !magn) return -1;
    CtxScope scope(h->ctx);
    if (!scope.ok) return -2;
    for (int c = 0; c < 3; ++c)
        if (!ck(cuMemcpyDtoH(magn + c * h->num, h->mag[c], h->num * sizeof(double)), "D2H")) return -3;
    return 0;
}

}  // extern "C"
