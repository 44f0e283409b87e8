// Host check of the certification rule (solver.cuh certify_kernel).
//
// One directional sweep is restated on the host: every node, in an order in
// which its upstream neighbours (r+1 below, and the lateral sides the sweep
// comes from) come first, is computed once by the solver's node update
// (stencil.cuh fm_update) from an unset field above a fixed bottom face.  The
// rule then marks the nodes a recomputation could change; every node it
// clears is recomputed from the final field and must give the same bits.
// Random slowness models, plane-wave bottom faces, sweep directions (right
// or wrong for the wave) and both orders, in both precisions.
//
//   g++ -O2 -std=c++17 -ffp-contract=off certify_check.cpp -o check && ./check [grids]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "../parallel-fast-marching-method_gb300/csrc/stencil.cuh"

namespace {

using fm3dt::Lim;
using fm3dt::Spacing;

template <typename R>
uint64_t bits(R v)
{
    uint64_t b = 0;
    std::memcpy(&b, &v, sizeof(R));
    return b;
}

template <typename R>
struct Grid {
    int nr, nx, nz;
    std::vector<R> T, s;
    R hr, hx, hz;
    int order2;
    size_t at(int r, int x, int z) const { return ((size_t)r * nx + x) * nz + z; }
    bool in(int r, int x, int z) const { return r >= 0 && r < nr && x >= 0 && x < nx && z >= 0 && z < nz; }
    R get(int r, int x, int z) const { return in(r, x, z) ? T[at(r, x, z)] : Lim<R>::inf(); }
    R update(int r, int x, int z) const
    {
        R t1[6], t2[6];
        const int dr[6] = {-1, 1, 0, 0, 0, 0}, dx[6] = {0, 0, -1, 1, 0, 0}, dz[6] = {0, 0, 0, 0, -1, 1};
        unsigned inb = 0;
        for (int d = 0; d < 6; ++d) {
            t1[d] = get(r + dr[d], x + dx[d], z + dz[d]);
            t2[d] = get(r + 2 * dr[d], x + 2 * dx[d], z + 2 * dz[d]);
            if (in(r + dr[d], x + dx[d], z + dz[d])) inb |= 1u << d;
        }
        Spacing<R> sp;
        sp.h[0] = hr; sp.h[1] = hx; sp.h[2] = hz;
        for (int a = 0; a < 3; ++a) sp.w[a] = R(1) / (sp.h[a] * sp.h[a]);
        return fm3dt::fm_update<R>(s[at(r, x, z)], t1, t2, inb, sp, order2);
    }
};

// the rule of certify_kernel: sx, sz are the lateral directions the sweep
// runs toward (+1 / -1); up (r-1) is always downstream
template <typename R>
bool certified(const Grid<R> &g, int r, int x, int z, int sx, int sz)
{
    const R INF = Lim<R>::inf();
    const R margin = R(1.0 / 32.0);
    const R T = g.get(r, x, z);
    const R td = g.get(r + 1, x, z), txu = g.get(r, x - sx, z), tzu = g.get(r, x, z - sz);
    const R tu = fm3dt::fm_min<R>(td, fm3dt::fm_min<R>(txu, tzu));
    if (!(T < INF && tu < INF)) return false;
    const R B = T - tu;
    const R hi = B + B * margin, lo = B - B * margin;
    auto down_ok = [&](R t1, R t2) { return (t1 - tu) >= hi && !(g.order2 && t2 < t1); };
    if (!down_ok(g.get(r - 1, x, z), g.get(r - 2, x, z))) return false;
    if (!down_ok(g.get(r, x + sx, z), g.get(r, x + 2 * sx, z))) return false;
    if (!down_ok(g.get(r, x, z + sz), g.get(r, x, z + 2 * sz))) return false;
    if (g.order2) {
        if (g.in(r + 1, x, z) && !((td - tu) < lo) && g.get(r + 2, x, z) < td) return false;
        if (g.in(r, x - sx, z) && !((txu - tu) < lo) && g.get(r, x - 2 * sx, z) < txu) return false;
        if (g.in(r, x, z - sz) && !((tzu - tu) < lo) && g.get(r, x, z - 2 * sz) < tzu) return false;
    }
    return true;
}

template <typename R>
void run(int ngrids, unsigned seed, long &nodes, long &cleared, long &bad)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (int it = 0; it < ngrids; ++it) {
        Grid<R> g;
        g.nr = 10 + (int)(rng() % 14);
        g.nx = 6 + (int)(rng() % 14);
        g.nz = 6 + (int)(rng() % 14);
        g.hr = R(2.0 + U(rng) * 2.0);
        g.hx = R(g.hr * (1.0 + U(rng) * 2.5));
        g.hz = R(g.hr * (1.0 + U(rng) * 2.5));
        g.order2 = (int)(rng() & 1);
        const size_t n = (size_t)g.nr * g.nx * g.nz;
        g.T.assign(n, Lim<R>::inf());
        g.s.resize(n);
        const double rough = (it % 3 == 0) ? 0.15 : 0.03;
        for (size_t q = 0; q < n; ++q) g.s[q] = R((1.0 / 8.0) * (1.0 + rough * (2.0 * U(rng) - 1.0)));
        // plane wave on the bottom face (fixed), times as offsets from its earliest node
        const double az = U(rng) * 2.0 * M_PI, p = 0.02 + U(rng) * 0.08;
        double tmin = 1e300;
        std::vector<double> bot((size_t)g.nx * g.nz);
        for (int x = 0; x < g.nx; ++x)
            for (int z = 0; z < g.nz; ++z) {
                bot[(size_t)x * g.nz + z] = p * (std::cos(az) * x * g.hx + std::sin(az) * z * g.hz);
                tmin = std::min(tmin, bot[(size_t)x * g.nz + z]);
            }
        for (int x = 0; x < g.nx; ++x)
            for (int z = 0; z < g.nz; ++z) g.T[g.at(g.nr - 1, x, z)] = R(bot[(size_t)x * g.nz + z] - tmin);
        // the sweep: toward the wave's lateral direction most of the time, the
        // other way sometimes
        int sx = std::cos(az) >= 0 ? 1 : -1, sz = std::sin(az) >= 0 ? 1 : -1;
        if (rng() % 4 == 0) sx = -sx;
        if (rng() % 4 == 0) sz = -sz;
        for (int r = g.nr - 2; r >= 0; --r)
            for (int i = 0; i < g.nx; ++i)
                for (int k = 0; k < g.nz; ++k) {
                    const int x = sx > 0 ? i : g.nx - 1 - i, z = sz > 0 ? k : g.nz - 1 - k;
                    g.T[g.at(r, x, z)] = g.update(r, x, z);
                }
        for (int r = 0; r < g.nr - 1; ++r)
            for (int x = 0; x < g.nx; ++x)
                for (int z = 0; z < g.nz; ++z) {
                    ++nodes;
                    if (!certified(g, r, x, z, sx, sz)) continue;
                    ++cleared;
                    if (bits(g.update(r, x, z)) != bits(g.get(r, x, z))) {
                        if (bad < 5)
                            std::printf("changed: grid %d node (%d,%d,%d) %.9g -> %.9g\n", it, r, x, z,
                                        (double)g.get(r, x, z), (double)g.update(r, x, z));
                        ++bad;
                    }
                }
    }
}

}  // namespace

int main(int argc, char **argv)
{
    const int ngrids = argc > 1 ? std::atoi(argv[1]) : 300;
    long nf = 0, cf = 0, bf = 0, nd = 0, cd = 0, bd = 0;
    run<float>(ngrids, 11, nf, cf, bf);
    run<double>(ngrids, 12, nd, cd, bd);
    std::printf("float: %ld nodes, %ld cleared, %ld changed; double: %ld nodes, %ld cleared, %ld changed\n",
                nf, cf, bf, nd, cd, bd);
    return (bf || bd || cf < nf / 4 || cd < nd / 4) ? 1 : 0;
}
