// Host replay of the reference's pulse schedules (no GPU needed).
//
// The reference decides at every step i, with currentTime = i*dTime, whether
// a pulse falls in the window [t, t + dTime) and applies it to the whole
// field (Sequence, src/NmrRelaxationSolve.cpp:2610-2679, CPU path; and
// Sequence_gpu, cpp:2681-3146, GPU path, which adds NSEQUENCE 5, 9, 98, 99
// and differs from the CPU one for CPMG and PFG). Here the same window tests,
// in the same floating-point expressions, produce a pulse list that the
// step kernel applies on the device.
#include <vector>

#include "../../include/bt.h"

namespace {

const double kPi = 3.1415926535897932384626433832795028841971;

struct Out {
    std::vector<bt_pulse> v;
    void add(long long step, int flag, double param, double ax, double ay, double az) {
        bt_pulse p{};
        p.step = step;
        p.flag = flag;
        p.param = param;
        p.axis[0] = ax;
        p.axis[1] = ay;
        p.axis[2] = az;
        v.push_back(p);
    }
};

inline bool in_window(double t, double start, double dt) { return (t < start + dt) && (t >= start); }

}  // namespace

extern "C" int bt_sequence_schedule(const bt_sequence_params* sp, long long nsteps, bt_pulse* out, int cap,
                                    int* count) {
    if (!sp || nsteps < 0 || cap < 0 || (cap > 0 && !out)) return BT_E_ARG;
    const double dt = sp->dt, T1 = sp->time1, T2 = sp->time2;
    const double* d = sp->direction;
    const double gp = sp->gradient_pulse;
    const double* mg = sp->multiple_gradients;
    const int seq = sp->n_sequence;
    const bool gpu = sp->gpu_variant != 0;
    int f1 = 0, f2 = 0, f3 = 0, f4 = 0, f5 = 0;
    Out o;
    for (long long i = 0; i < nsteps; ++i) {
        const double t = i * dt;
        if (seq == 0) {
            if ((t < dt) && (t >= 0.0)) o.add(i, 2, 0.5 * kPi, d[2], d[0], d[1]);
        } else if (seq == 1) {
            if ((t < dt) && (t >= 0.0)) o.add(i, 2, 0.5 * kPi, d[2], d[0], d[1]);
            const int n180 = gpu ? 20 : 100;
            for (int q = 0; q < n180; ++q)
                if ((t < (2 * q + 1) * T1 + dt) && (t >= (2 * q + 1) * T1)) o.add(i, 2, kPi, d[2], d[0], d[1]);
        } else if (seq == 2) {
            const double s90 = gpu ? -d[2] : d[2];
            if ((t < dt) && (t >= 0.0) && f1 == 0) { o.add(i, 2, 0.5 * kPi, s90, d[0], d[1]); f1 = 1; }
            if (in_window(t, T1, dt) && f2 == 0) { o.add(i, 1, gp, d[0], d[1], d[2]); f2 = 1; }
            if ((t < 2.0 * T1 + dt) && (t >= 2.0 * T1) && f3 == 0) { o.add(i, 2, 0.5 * kPi, d[2], d[0], d[1]); f3 = 1; }
            if ((t < 2.0 * T1 + T2 + dt) && (t >= 2.0 * T1 + T2) && f4 == 0) {
                o.add(i, 2, 0.5 * kPi, s90, d[0], d[1]);
                f4 = 1;
            }
            if ((t < 3.0 * T1 + T2 + dt) && (t >= 3.0 * T1 + T2) && f5 == 0) { o.add(i, 1, gp, d[0], d[1], d[2]); f5 = 1; }
        } else if (gpu && seq == 9) {
            if ((t < dt) && (t >= 0.0) && f1 == 0) { o.add(i, 2, 0.5 * kPi, d[2], d[0], d[1]); f1 = 1; }
            if (in_window(t, T1, dt) && f2 == 0) { o.add(i, 1, gp, d[0], d[1], d[2]); f2 = 1; }
            if ((t < T1 + T2 / 2 + dt) && (t >= T1 + T2 / 2) && f3 == 0) { o.add(i, 2, kPi, d[2], d[0], d[1]); f3 = 1; }
            if ((t < T2 + T1 + dt) && (t >= T2 + T1) && f4 == 0) { o.add(i, 1, gp, d[0], d[1], d[2]); f4 = 1; }
        } else if (gpu && seq == 5) {
            if ((t < dt) && (t >= 0.0)) o.add(i, 2, kPi, d[2], d[0], d[1]);
        } else if (gpu && seq == 99) {
            if ((t < dt) && (t >= 0.0) && f1 == 0) f1 = 1;
            if (in_window(t, T1, dt) && f2 == 0) { o.add(i, 3, 1.0, mg[0], mg[1], mg[2]); f2 = 1; }
            if ((t < T1 + T2 / 2 + dt) && (t >= T1 + T2 / 2) && f3 == 0) f3 = 1;
            if ((t < T2 + T1 + dt) && (t >= T2 + T1) && f4 == 0) { o.add(i, 3, 1.0, -mg[0], -mg[1], -mg[2]); f4 = 1; }
        } else if (gpu && seq == 98) {
            if ((t < dt) && (t >= 0.0) && f1 == 0) { o.add(i, 2, 0.5 * kPi, 0.0, -1.0, 0.0); f1 = 1; }
            if (in_window(t, T1, dt) && f2 == 0) { o.add(i, 3, 1.0, mg[0], mg[1], mg[2]); f2 = 1; }
            if ((t < T1 + T2 / 2 + dt) && (t >= T1 + T2 / 2) && f3 == 0) { o.add(i, 2, kPi, 0.0, 0.0, 1.0); f3 = 1; }
            if ((t < T2 + T1 + dt) && (t >= T2 + T1) && f4 == 0) { o.add(i, 3, 1.0, mg[0], mg[1], mg[2]); f4 = 1; }
        }
    }
    if (count) *count = (int)o.v.size();
    for (int q = 0; q < (int)o.v.size() && q < cap; ++q) out[q] = o.v[q];
    return BT_OK;
}
