// Arithmetic count of the oracle's P0 pair functions (TEST INFRASTRUCTURE,
// not the product): p0_oracle.c compiled with `double` replaced by a type
// that counts every add/subtract, multiply, divide and special function
// (sqrt, log, atan2) it executes. This gives the algorithmic work per
// (observer, source) pair of the reference's formulas as the oracle states
// them (src/mbem/kernels/tri_kernels.py), independent of the CUDA code:
// FLOPs = adds + multiplies (an FMA counts as its two), with divides and
// special functions reported beside them.
//
// Build: g++ -O1 -std=c++17 -fPIC -shared oracle/flop_count.cpp -o
// oracle/_build/libflop_count.so (oracle/flop_count.py does it).
#include <math.h>
#include <stdint.h>
#include <string.h>

namespace {

struct Counts {
    long long add, mul, div, special;
};
Counts g_n = {0, 0, 0, 0};

struct Flop {
    double v;
    Flop() = default;
    Flop(double x) : v(x) {}
};

inline Flop operator+(Flop a, Flop b) { g_n.add++; return Flop(a.v + b.v); }
inline Flop operator-(Flop a, Flop b) { g_n.add++; return Flop(a.v - b.v); }
inline Flop operator*(Flop a, Flop b) { g_n.mul++; return Flop(a.v * b.v); }
inline Flop operator/(Flop a, Flop b) { g_n.div++; return Flop(a.v / b.v); }
inline Flop operator-(Flop a) { return Flop(-a.v); }
inline Flop& operator+=(Flop& a, Flop b) { a = a + b; return a; }
inline Flop& operator-=(Flop& a, Flop b) { a = a - b; return a; }
inline Flop& operator*=(Flop& a, Flop b) { a = a * b; return a; }
inline Flop& operator/=(Flop& a, Flop b) { a = a / b; return a; }
inline bool operator<(Flop a, Flop b) { return a.v < b.v; }
inline bool operator>(Flop a, Flop b) { return a.v > b.v; }
inline bool operator<=(Flop a, Flop b) { return a.v <= b.v; }
inline bool operator>=(Flop a, Flop b) { return a.v >= b.v; }
inline bool operator==(Flop a, Flop b) { return a.v == b.v; }
inline bool operator!=(Flop a, Flop b) { return a.v != b.v; }
inline Flop sqrt(Flop a) { g_n.special++; return Flop(::sqrt(a.v)); }
inline Flop log(Flop a) { g_n.special++; return Flop(::log(a.v)); }
inline Flop atan2(Flop a, Flop b) { g_n.special++; return Flop(::atan2(a.v, b.v)); }
inline Flop fabs(Flop a) { return Flop(::fabs(a.v)); }

}  // namespace

#define double Flop
#include "p0_oracle.c"
#undef double

extern "C" {

// Walks every (observer f, source s) pair of the arrays through one pair
// function and returns the counts summed over the pairs:
// kind 0 T block (the six basis blocks and their t_coeffs combination),
// 1 U block, 2 DD stress, 3 Kelvin stress, 4 eigenstress, 5 solid angle.
// counts[4] = adds, multiplies, divides, special functions; the return
// value is the number of pairs walked (degenerate sources skipped).
long long flop_count(int kind, const double* x_field, int64_t Nf, const double* tri_verts, const double* normals,
                     const double* eps_arr, int64_t Ns, long long* counts) {
    g_n = Counts{0, 0, 0, 0};
    long long pairs = 0;
    const double mu = 1.0, lam = 1.0, nu = 0.25;
    const double cs[6] = {1.0, 0.5, 0.25, 0.125, 0.0625, 0.03125};
    for (int64_t s = 0; s < Ns; s++) {
        Flop tv[9], nrm[3], ex[3], ey[3], nh[3];
        for (int k = 0; k < 9; k++) tv[k] = Flop(tri_verts[9 * s + k]);
        for (int k = 0; k < 3; k++) nrm[k] = Flop(normals[3 * s + k]);
        const Counts before = g_n;
        const int ok = tri_frame(tv, ex, ey, nh);
        // the per-source frame is set up once a source, not once a pair
        g_n = before;
        if (!ok) continue;
        const Flop eps(eps_arr[s]);
        for (int64_t f = 0; f < Nf; f++) {
            Flop obs[3] = {Flop(x_field[3 * f]), Flop(x_field[3 * f + 1]), Flop(x_field[3 * f + 2])};
            pairs++;
            if (kind == 0) {
                Flop blk[6][3][3];
                t_basis_pair(tv, ex, ey, nh, nrm, obs, eps, blk);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        Flop m = Flop(cs[0]) * blk[0][i][j];
                        for (int b = 1; b < 6; b++) m = m + Flop(cs[b]) * blk[b][i][j];
                    }
            } else if (kind == 1) {
                Flop blk[3][3][3];
                u_basis_pair(tv, ex, ey, nh, obs, eps, blk);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        Flop m = Flop(cs[0]) * blk[0][i][j];
                        for (int b = 1; b < 3; b++) m = m + Flop(cs[b]) * blk[b][i][j];
                    }
            } else if (kind == 2) {
                Flop H[3][3][3];
                dd_stress_pair(tv, ex, ey, nh, nrm, obs, eps, Flop(mu), Flop(nu), Flop(lam), H);
            } else if (kind == 3) {
                Flop H[3][3][3];
                kelvin_stress_pair(tv, ex, ey, nh, obs, eps, Flop(mu), Flop(nu), Flop(lam), H);
            } else if (kind == 4) {
                Flop H[3][3][3];
                eigenstress_pair(tv, ex, ey, nh, nrm, obs, eps, Flop(mu), Flop(lam), H);
            } else {
                (void)solid_angle(tv, obs[0], obs[1], obs[2]);
            }
        }
    }
    counts[0] = g_n.add;
    counts[1] = g_n.mul;
    counts[2] = g_n.div;
    counts[3] = g_n.special;
    return pairs;
}

}  // extern "C"
