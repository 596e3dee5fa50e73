// point_source.cuh -- the point source and the receiver of the acoustic programs
// 3d/weno4/point_source and 2d/weno4/line_source, host side.
//
// The source is the derivative-of-Gaussian wavelet of source.c:11-17,
//   Source(t) = -2 (t - t0) f0^2 exp(-f0^2 (t - t0)^2),  t0 = 4 / f0,
// added to the u_t equation of one cell as Source(t) / h^3 (3D, rhs_function.c:337-339)
// or Source(t) / h^2 (2D, rhs_function.c:244-246) at the time t of every RHS
// evaluation.  The receiver records u of one cell at every RHS evaluation
// (rhs_function.c:342-346 / :249-253 print it to results/p.dat).
//
// Source(t) is evaluated here, on the host, with the C library's exp and the reference's
// operation order, once per RHS evaluation; the kernel only adds the scaled value to the
// one cell, so the GPU's RHS equals the reference's bit for bit wherever the rest of it
// does.  The receiver's value is written by the update kernel into a device trace slot.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <vector>

namespace hype {

struct PointSource {
    bool src_on = false;
    long long src_cell = -1;  // linear index of the source cell in the owned grid
    double f0 = 0.0;
    double scale = 0.0;       // 1/h^3 or 1/h^2, as the reference computes it
    bool rec_on = false;
    long long rec_cell = -1;
    double* trace = nullptr;  // device, capacity values of u at the receiver
    int capacity = 0;
    long long count = 0;      // RHS evaluations seen since the receiver was set
    std::vector<double> times;

    // Source(t) / h^dim (source.c:11-17 times r1_h3 / r1_h2)
    double value(double t) const {
        const double t0 = 4.0 / f0;
        return -2.0 * (t - t0) * f0 * f0 * exp(-1.0 * f0 * f0 * (t - t0) * (t - t0)) * scale;
    }

    // the device slot the next RHS evaluation at time t writes u of the receiver to
    // (nullptr when the receiver is off or the trace is full)
    double* record(double t) {
        if (!rec_on) return nullptr;
        double* slot = count < capacity ? trace + count : nullptr;
        if (count < capacity) times.push_back(t);
        ++count;
        return slot;
    }

    void release() {
        if (trace) cudaFree(trace);
        trace = nullptr;
        capacity = 0;
    }
};

// the arguments one update-kernel launch gets
struct SourceArgs {
    long long src_cell;  // -1: no source
    double src_val;
    long long rec_cell;  // -1: no receiver slot
    double* slot;
};

inline SourceArgs source_args(PointSource& ps, double t) {
    SourceArgs s{-1, 0.0, -1, nullptr};
    if (ps.src_on) {
        s.src_cell = ps.src_cell;
        s.src_val = ps.value(t);
    }
    double* slot = ps.record(t);
    if (slot) {
        s.rec_cell = ps.rec_cell;
        s.slot = slot;
    }
    return s;
}

}  // namespace hype
