/*
 * build_race.cpp -- the threaded RSS hierarchy build under a sanitizer
 * (ThreadSanitizer or AddressSanitizer, chosen at compile time): builds the
 * triangle soup in argv[1] (int32 count, then count x 9 doubles) once on the
 * calling thread and once with argv[2] threads, and compares every byte of
 * the node, OBB, triangle and shadow records.  Exit 0 when they match.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../c2a_gb300/csrc/host/bvh_build.h"

template <class V> static bool same(const V &a, const V &b)
{
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(a[0])) == 0;
}

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1 || n <= 0) return 2;
    std::vector<double> tv(9 * (size_t)n);
    if (std::fread(tv.data(), sizeof(double), tv.size(), f) != tv.size()) return 2;
    std::fclose(f);
    const int threads = std::atoi(argv[2]);

    c2a::BuiltModel one, many;
    if (c2a::build_rss_model(n, tv.data(), nullptr, nullptr, one) != 0) return 3;
    c2a::BuildThreads budget(threads - 1);
    if (c2a::build_rss_model(n, tv.data(), nullptr, nullptr, many, &budget) != 0) return 3;
    // every thread taken from the budget was given back
    int back = 0;
    while (budget.take()) back++;
    const bool ok = same(one.nodes, many.nodes) && same(one.obbs, many.obbs) && same(one.tris, many.tris) &&
                    same(one.snodes, many.snodes) && same(one.stris, many.stris) && one.depth == many.depth &&
                    one.shadow_ok == many.shadow_ok && back == threads - 1;
    std::printf("%s: %d triangles, %d threads, depth %d, budget back %d\n", ok ? "same" : "DIFFERENT", n, threads,
                many.depth, back);
    return ok ? 0 : 1;
}
