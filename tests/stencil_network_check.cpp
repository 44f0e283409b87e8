// Host checks.  (1) The solver's node update (stencil.cuh fm_update, as optimised:
// lateral pairs sorted once per two octants, hardware min/max, outside
// octants masked by a select) against a plain restatement of the same
// update (every octant sorted by a full three-comparator stable network,
// outside octants skipped), bit for bit, on random inputs with ties, unset
// neighbours, and +inf or NaN outside the grid as the kernels stage them.
// (2) The main sweep's upstream-only update against fm_update with its
// downstream neighbours unset, bit for bit.
//
//   g++ -O2 -std=c++17 -ffp-contract=off stencil_network_check.cpp -o check && ./check [cases]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "../parallel-fast-marching-method_gb300/csrc/stencil.cuh"

namespace {

using fm3dt::Fast;
using fm3dt::Lim;
using fm3dt::Spacing;

template <typename R>
R plain_update(R s, const R t1[6], const R t2[6], unsigned inb, const Spacing<R> &sp, int order2)
{
    const R INF = Lim<R>::inf();
    R tmin = INF;
    for (int d = 0; d < 6; ++d)
        if (((inb >> d) & 1u) && t1[d] < tmin) tmin = t1[d];
    if (!(tmin < INF)) return INF;
    const R s2 = s * s;
    R key[6], e[6], g[6], w[6];
    for (int d = 0; d < 6; ++d) {
        const int a = d >> 1;
        const bool o2 = order2 && (t2[d] < t1[d]);
        const R dt = t1[d] - tmin;
        key[d] = ((inb >> d) & 1u) ? dt : INF;
        e[d] = o2 ? fm3dt::fm_fma<R>(t1[d] - t2[d], R(1.0 / 3.0), dt) : dt;
        g[d] = o2 ? sp.h[a] * R(2.0 / 3.0) : sp.h[a];
        w[d] = o2 ? sp.w[a] * R(2.25) : sp.w[a];
    }
    R best = INF;
    for (int o = 0; o < 8; ++o) {
        const int dir[3] = {(o >> 2) & 1, 2 + ((o >> 1) & 1), 4 + (o & 1)};
        if (!(((inb >> dir[0]) & (inb >> dir[1]) & (inb >> dir[2])) & 1u)) continue;
        R k[3], ee[3], gg[3], ww[3];
        for (int i = 0; i < 3; ++i) {
            k[i] = key[dir[i]]; ee[i] = e[dir[i]]; gg[i] = g[dir[i]]; ww[i] = w[dir[i]];
        }
        // stable: swap only when the later key is strictly smaller
        const int net[3][2] = {{0, 1}, {1, 2}, {0, 1}};
        for (const auto &p : net) {
            const int i = p[0], j = p[1];
            if (k[j] < k[i]) {
                R q;
                q = k[i]; k[i] = k[j]; k[j] = q;
                q = ee[i]; ee[i] = ee[j]; ee[j] = q;
                q = gg[i]; gg[i] = gg[j]; gg[j] = q;
                q = ww[i]; ww[i] = ww[j]; ww[j] = q;
            }
        }
        if (!(k[0] < INF)) continue;
        R x = fm3dt::fm_fma<R>(s, gg[0], ee[0]);
        if (k[1] < x) {
            R a = ww[0] + ww[1];
            const R we0 = ww[0] * ee[0], we1 = ww[1] * ee[1];
            R b = we0 + we1;
            R c = fm3dt::fm_fma<R>(we0, ee[0], fm3dt::fm_fma<R>(we1, ee[1], -s2));
            R disc = fm3dt::fm_fma<R>(b, b, -(a * c));
            x = Fast<R>::div(b + Fast<R>::sqrt(disc > R(0) ? disc : R(0)), a);
            if (k[2] < x) {
                const R we2 = ww[2] * ee[2];
                a += ww[2];
                b += we2;
                c = fm3dt::fm_fma<R>(we2, ee[2], c);
                disc = fm3dt::fm_fma<R>(b, b, -(a * c));
                x = Fast<R>::div(b + Fast<R>::sqrt(disc > R(0) ? disc : R(0)), a);
            }
        }
        if (x < best) best = x;
    }
    return tmin + best;
}

template <typename R>
uint64_t bits(R v)
{
    uint64_t b = 0;
    std::memcpy(&b, &v, sizeof(R));
    return b;
}

template <typename R>
long run(long n, unsigned seed)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const R INF = Lim<R>::inf();
    long bad = 0;
    for (long it = 0; it < n; ++it) {
        R t1[6], t2[6];
        const int levels = (int)(rng() % 4);   // 0: continuous, else a few values (ties)
        for (int d = 0; d < 6; ++d) {
            const double v1 = levels ? (double)(rng() % (2 + levels)) * 0.5 : U(rng) * 3.0;
            const double v2 = levels ? (double)(rng() % (2 + levels)) * 0.5 : U(rng) * 3.0;
            t1[d] = (rng() % 13 == 0) ? INF : R(v1);
            t2[d] = (rng() % 9 == 0) ? INF : R(v2);
        }
        const unsigned inb = (rng() % 3 == 0) ? (unsigned)(rng() & 63) : 63u;
        for (int d = 0; d < 6; ++d)
            if (!((inb >> d) & 1u)) {
                t1[d] = (rng() & 1) ? INF : R(NAN);
                t2[d] = (rng() & 1) ? INF : R(NAN);
            }
        Spacing<R> sp;
        for (int a = 0; a < 3; ++a) {
            const double h = 0.5 + U(rng) * 2.5;
            sp.h[a] = R(h);
            sp.w[a] = R(1.0 / (h * h));
        }
        const R s = R(0.1 + U(rng));
        const int order2 = (int)(rng() & 1);
        const R want = plain_update<R>(s, t1, t2, inb, sp, order2);
        const R got = fm3dt::fm_update<R>(s, t1, t2, inb, sp, order2);
        if (bits(want) != bits(got)) {
            if (bad < 5) std::printf("mismatch: %.9g vs %.9g\n", (double)want, (double)got);
            ++bad;
        }
    }
    return bad;
}

// The main sweep's node update (fm_update_upstream, only the three upstream
// neighbours) against fm_update with +inf at the three downstream neighbours,
// for every sweep direction: random upstream values with ties and unset
// ones, random second neighbours (downstream ones too), neighbours outside
// the grid (+inf there, as the streaming sweep stages them), both orders.
template <typename R>
long run_upstream(long n, unsigned seed)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const R INF = Lim<R>::inf();
    long bad = 0;
    for (long it = 0; it < n; ++it) {
        const bool sx = rng() & 1, sz = rng() & 1;
        const int dX = sx ? 2 : 3, dZ = sz ? 4 : 5;      // upstream lateral directions
        const int levels = (int)(rng() % 4);
        R t1[6], t2[6];
        for (int d = 0; d < 6; ++d) {
            const double v1 = levels ? (double)(rng() % (2 + levels)) * 0.5 : U(rng) * 3.0;
            const double v2 = levels ? (double)(rng() % (2 + levels)) * 0.5 : U(rng) * 3.0;
            t1[d] = (rng() % 13 == 0) ? INF : R(v1);
            t2[d] = (rng() % 9 == 0) ? INF : R(v2);
        }
        // downstream neighbours unset
        t1[0] = INF;
        t1[dX ^ 1] = INF;
        t1[dZ ^ 1] = INF;
        unsigned inb = 63u;
        if (rng() % 3 == 0) inb = (unsigned)(rng() & 63);
        for (int d = 0; d < 6; ++d)
            if (!((inb >> d) & 1u)) {
                t1[d] = INF;
                t2[d] = INF;
            }
        Spacing<R> sp;
        for (int a = 0; a < 3; ++a) {
            const double h = 0.5 + U(rng) * 2.5;
            sp.h[a] = R(h);
            sp.w[a] = R(1.0 / (h * h));
        }
        const R s = R(0.1 + U(rng));
        const int order2 = (int)(rng() & 1);
        const R want = fm3dt::fm_update<R>(s, t1, t2, inb, sp, order2);
        const R got = fm3dt::fm_update_upstream<R>(
            s, t1[1], t2[1], t1[dX], t2[dX], t1[dZ], t2[dZ], (inb >> 1) & 1u, inb & 1u, (inb >> dX) & 1u,
            (inb >> (dX ^ 1)) & 1u, (inb >> dZ) & 1u, (inb >> (dZ ^ 1)) & 1u, sp, order2);
        if (bits(want) != bits(got)) {
            if (bad < 5) std::printf("upstream mismatch: %.9g vs %.9g\n", (double)want, (double)got);
            ++bad;
        }
    }
    return bad;
}

}  // namespace

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 200000;
    const long bf = run<float>(n, 1), bd = run<double>(n, 2);
    std::printf("float mismatches %ld / %ld, double mismatches %ld / %ld\n", bf, n, bd, n);
    const long uf = run_upstream<float>(n, 3), ud = run_upstream<double>(n, 4);
    std::printf("upstream float mismatches %ld / %ld, upstream double mismatches %ld / %ld\n", uf, n, ud, n);
    return (bf || bd || uf || ud) ? 1 : 0;
}
