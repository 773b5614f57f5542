// gi_host.cpp -- host-side parts of libgi.so: seeded initial-condition
// generators.  Compiled with -ffp-contract=off and only +, -, *, /, sqrt
// (all IEEE-exact or correctly rounded), so a given seed produces the same
// bodies on x86-64 and aarch64 hosts.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/gi_api.h"
#include "gi_host.h"

namespace {

// Uniform point in the unit ball by rejection from the cube (no
// transcendental functions, so bit-identical across hosts).
void unit_ball(gi_host::Rng &g, double &x, double &y, double &z)
{
    for (;;) {
        x = 2.0 * g.uniform() - 1.0;
        y = 2.0 * g.uniform() - 1.0;
        z = 2.0 * g.uniform() - 1.0;
        if (x * x + y * y + z * z <= 1.0) return;
    }
}

}  // namespace

extern "C" int gi_ic_uniform_ball(unsigned long long seed, int n, double radius,
                                  double fe_radius_fraction, float mass_fe, float mass_si,
                                  float tag_fe, float tag_si, float *pos, float *vel,
                                  int *nfe_out)
{
    if (n < 0 || !(radius > 0.0) || !pos || !vel || !nfe_out) return GI_ERR_INVALID_ARG;
    gi_host::Rng g(seed);
    std::vector<float> fe, si;
    fe.reserve(3 * (size_t)n);
    si.reserve(3 * (size_t)n);
    const double rfe2 = fe_radius_fraction * fe_radius_fraction;
    for (int k = 0; k < n; ++k) {
        double x, y, z;
        unit_ball(g, x, y, z);
        std::vector<float> &dst = (x * x + y * y + z * z < rfe2) ? fe : si;
        dst.push_back((float)(radius * x));
        dst.push_back((float)(radius * y));
        dst.push_back((float)(radius * z));
    }
    const int nfe = (int)(fe.size() / 3);
    for (int k = 0; k < n; ++k) {
        const bool isfe = k < nfe;
        const float *src = isfe ? &fe[3 * (size_t)k] : &si[3 * (size_t)(k - nfe)];
        float *p = pos + 4 * (size_t)k, *v = vel + 4 * (size_t)k;
        p[0] = src[0]; p[1] = src[1]; p[2] = src[2];
        p[3] = isfe ? tag_fe : tag_si;
        v[0] = v[1] = v[2] = 0.0f;
        v[3] = isfe ? mass_fe : mass_si;
    }
    *nfe_out = nfe;
    return GI_OK;
}

extern "C" int gi_ic_lattice(unsigned long long seed, int n, double spacing, double jitter,
                             double vel_sigma, int nfe, float mass_fe, float mass_si,
                             float *pos, float *vel)
{
    if (n < 0 || nfe < 0 || nfe > n || !pos || !vel) return GI_ERR_INVALID_ARG;
    gi_host::Rng g(seed);
    int side = 1;
    while ((long long)side * side * side < n) ++side;
    for (int k = 0; k < n; ++k) {
        const int ix = k % side, iy = (k / side) % side, iz = k / (side * side);
        float *p = pos + 4 * (size_t)k, *v = vel + 4 * (size_t)k;
        p[0] = (float)(spacing * ix + jitter * (2.0 * g.uniform() - 1.0));
        p[1] = (float)(spacing * iy + jitter * (2.0 * g.uniform() - 1.0));
        p[2] = (float)(spacing * iz + jitter * (2.0 * g.uniform() - 1.0));
        p[3] = (k < nfe) ? 0.0f : 1.0f;
        // Irwin-Hall approximation of a normal: sum of 12 uniforms - 6.
        for (int a = 0; a < 3; ++a) {
            double s = -6.0;
            for (int m = 0; m < 12; ++m) s += g.uniform();
            v[a] = (float)(vel_sigma * s);
        }
        v[3] = (k < nfe) ? mass_fe : mass_si;
    }
    return GI_OK;
}
