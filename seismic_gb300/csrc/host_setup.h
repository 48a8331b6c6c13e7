// host_setup.h -- host restatements of the reference's per-geometry constants,
// shared by every entry point that builds a sweep (engine.cu, noalloc.cu) so
// that their records agree bitwise.  Both run once per engine / call in FP64.
#pragma once
#include <cmath>
#include <vector>

namespace seis {

// Samples of the Ricker wavelet that can be non-zero: nw = 2 * (int(2.2 / f / dt) / 2) + 1
// (ricker(), core/seis_forward2.py:20-40).
inline int ricker_length(double freq, double dt)
{
    const int nw = (int)(2.2 / freq / dt);
    return 2 * (nw / 2) + 1;
}

// ricker() + expand_source() (core/seis_forward2.py:20-45): w(k) = (1 - 2b) e^-b with
// b = ((nc - k) f dt pi)^2, zero-padded to nt.  Returns nw, or -1 when nt < nw.
inline int host_ricker(double freq, double dt, int nt, std::vector<double>& w)
{
    const int nw = ricker_length(freq, dt);
    const int nc = nw / 2 + 1;
    if (nt < nw) return -1;
    w.assign(nt, 0.0);
    for (int k = 1; k <= nw; ++k) {
        const double a = (double)(nc - k) * freq * dt * M_PI;
        const double b = a * a;
        w[k - 1] = (1.0 - 2.0 * b) * std::exp(-b);
    }
    return nw;
}

// The 1-D sponge profile of AbcCoef2D (core/seis_forward2.py:46-59):
// d1[i] = kappa ((i dx) / a)^2, a = (nbc - 1) dx, kappa = 3 ln(1e7) / (2a).
inline void host_damp_1d(int nbc, double dx, std::vector<double>& d1)
{
    const double a = (nbc - 1) * dx;
    const double kappa = 3.0 * std::log(1e7) / (2.0 * a);
    d1.assign(nbc, 0.0);
    for (int i = 0; i < nbc; ++i) {
        const double r = (i * dx) / a;
        d1[i] = kappa * (r * r);
    }
}

// The profile mirrored onto the padded columns (dampx, `pitch` long) and rows
// (dampz, NZ long), zero on the interior; the corner rule (side bands cover
// every row) is applied where the kernels read them (damp_at, common.cuh).
inline void host_damp_profiles(int nbc, int nz, int nx, double dx, int pitch, int NZ, std::vector<double>& dampx,
                               std::vector<double>& dampz)
{
    std::vector<double> d1;
    host_damp_1d(nbc, dx, d1);
    dampx.assign(pitch, 0.0);
    dampz.assign(NZ, 0.0);
    for (int i = 0; i < nbc; ++i) {
        dampx[i] = d1[nbc - 1 - i];
        dampx[nx + nbc + i] = d1[i];
        dampz[i] = d1[nbc - 1 - i];
        dampz[nz + nbc + i] = d1[i];
    }
}

}  // namespace seis
