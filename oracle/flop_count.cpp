/*
 * flop_count.cpp -- the FP64 operation counts of the CA path, per node-pair
 * test and per leaf triangle test, taken from the oracle's own restatement
 * of the reference (c2a_port_geom.c, c2a_port_ca.c) compiled with a counting
 * double.  Test infrastructure only: the roofline's per-unit flop figures are
 * measured with it and a test checks them.
 *
 * Every +, -, * and / on a double is one operation, sqrt one; comparisons
 * are tallied apart and are not flops; fabs, negation and copies are free.
 * Operations go to the bucket of the innermost open scope (C2A_PORT_SCOPE in
 * the port): 1 a node-pair expansion (the two child transforms, both RSS
 * distances and motion bounds, the descent tests; C2A.cpp:1194-1354), 2 a
 * leaf triangle test (C2A.cpp:1155-1192), 3 contact enumeration at the TOC,
 * 0 everything else (motion integration, the CA loop).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../c2a_gb300/csrc/common/c2a_detmath.h"

namespace fc {
enum { ADD, MUL, DIV, SQRT, CMP, KINDS };
thread_local long long ops[4][KINDS];
thread_local int bucket = 0;
struct Scope {
    int prev;
    explicit Scope(int k) : prev(bucket) { bucket = k; }
    ~Scope() { bucket = prev; }
};
inline void tick(int kind) { ops[bucket][kind]++; }
} // namespace fc

struct CD {
    double v;
    CD() = default;
    constexpr CD(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    CD &operator+=(CD b) { fc::tick(fc::ADD); v += b.v; return *this; }
    CD &operator-=(CD b) { fc::tick(fc::ADD); v -= b.v; return *this; }
    CD &operator*=(CD b) { fc::tick(fc::MUL); v *= b.v; return *this; }
    CD &operator/=(CD b) { fc::tick(fc::DIV); v /= b.v; return *this; }
};
static_assert(sizeof(CD) == sizeof(double), "layout");
inline CD operator+(CD a, CD b) { fc::tick(fc::ADD); return a.v + b.v; }
inline CD operator-(CD a, CD b) { fc::tick(fc::ADD); return a.v - b.v; }
inline CD operator*(CD a, CD b) { fc::tick(fc::MUL); return a.v * b.v; }
inline CD operator/(CD a, CD b) { fc::tick(fc::DIV); return a.v / b.v; }
inline CD operator-(CD a) { return -a.v; }
inline bool operator<(CD a, CD b) { fc::tick(fc::CMP); return a.v < b.v; }
inline bool operator>(CD a, CD b) { fc::tick(fc::CMP); return a.v > b.v; }
inline bool operator<=(CD a, CD b) { fc::tick(fc::CMP); return a.v <= b.v; }
inline bool operator>=(CD a, CD b) { fc::tick(fc::CMP); return a.v >= b.v; }
inline bool operator==(CD a, CD b) { fc::tick(fc::CMP); return a.v == b.v; }
inline bool operator!=(CD a, CD b) { fc::tick(fc::CMP); return a.v != b.v; }
inline CD sqrt(CD a) { fc::tick(fc::SQRT); return ::sqrt(a.v); }
inline CD fabs(CD a) { return ::fabs(a.v); }
inline bool isnan(CD a) { return a.v != a.v; }
inline CD c2a_det_sin(CD x) { return c2a_det_sin(x.v); }
inline CD c2a_det_cos(CD x) { return c2a_det_cos(x.v); }
inline CD c2a_det_acos(CD x) { return c2a_det_acos(x.v); }

#define C2A_PORT_SCOPE(k) fc::Scope c2a_fc_scope_(k)
#define double CD
#include "c2a_port_geom.c"
#include "c2a_port_ca.c"
#undef double

/* Solves n queries (the port's batch layout: qint n x 4, poses n x 48) one
 * after another on the calling thread; ops_out receives 4 buckets x 5 kinds
 * (add/sub, mul, div, sqrt, compare), counts_out the summed num_bv_tests and
 * num_tri_tests.  Returns the number of rejected queries. */
extern "C" int c2a_fc_solve(const c2a_port_model *models, int num_models, const int *qint, const double *poses, int n,
                            const c2a_port_params *prm, long long *ops_out, long long *counts_out)
{
    memset(fc::ops, 0, sizeof(fc::ops));
    fc::bucket = 0;
    long long nbv = 0, ntri = 0;
    int bad = 0;
    const int slots = 64;
    c2a_port_contact *con = (c2a_port_contact *)malloc(sizeof(c2a_port_contact) * slots);
    for (int q = 0; q < n; q++) {
        const int *qi = qint + 4 * q;
        const CD *p = (const CD *)(poses + 48 * q);
        if (qi[0] < 0 || qi[0] >= num_models || qi[1] < 0 || qi[1] >= num_models) {
            bad++;
            continue;
        }
        c2a_port_result r;
        if (c2a_port_solve(&models[qi[0]], &models[qi[1]], p, p + 9, p + 12, p + 21, p + 24, p + 33, p + 36,
                           p + 45, qi[2], qi[3], prm, &r, con, slots) != 0)
            bad++;
        nbv += r.num_bv_tests;
        ntri += r.num_tri_tests;
    }
    free(con);
    memcpy(ops_out, fc::ops, sizeof(fc::ops));
    counts_out[0] = nbv;
    counts_out[1] = ntri;
    return bad;
}
