// The static queries of the C++ drop-in (C2A_Tolerance, C2A_Collide,
// C2A_Distance) on meshes and placements read from a binary file:
//   int32 num_meshes; per mesh int32 nv, nt, then nv x 3 doubles, nt x 3 int32;
//   int32 n; per query int32 a, b, then R (9 doubles), T (3 doubles), tolerance.
// Model a sits at the identity, model b at (R, T).  Prints, per query, one
// tolerance line "closer distance p1 p2 nbv ntri" (%.17g), one collide line
// "npairs nbv ntri id1 id2 ...", one distance line "distance t1 t2".
#include <cstdio>
#include <vector>

#include "c2a_gb300_cpp.h"

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    auto rd = [&](void *p, size_t sz, size_t n) { return std::fread(p, sz, n, f) == n; };
    int nm = 0;
    if (!rd(&nm, 4, 1)) return 3;
    std::vector<C2A_Model *> models;
    for (int m = 0; m < nm; m++) {
        int nv = 0, nt = 0;
        if (!rd(&nv, 4, 1) || !rd(&nt, 4, 1)) return 3;
        std::vector<double> v(3 * (size_t)nv);
        std::vector<int> t(3 * (size_t)nt);
        if (!rd(v.data(), 8, v.size()) || !rd(t.data(), 4, t.size())) return 3;
        C2A_Model *o = new C2A_Model();
        o->BeginModel();
        for (int i = 0; i < nt; i++)
            o->AddTri(&v[3 * t[3 * i]], &v[3 * t[3 * i + 1]], &v[3 * t[3 * i + 2]], i, t[3 * i], t[3 * i + 1],
                      t[3 * i + 2]);
        if (o->EndModel() != 0) return 4;
        models.push_back(o);
    }
    int n = 0;
    if (!rd(&n, 4, 1)) return 3;
    for (int k = 0; k < n; k++) {
        int ab[2];
        double Rv[9], T2[3], tol;
        if (!rd(ab, 4, 2) || !rd(Rv, 8, 9) || !rd(T2, 8, 3) || !rd(&tol, 8, 1)) return 3;
        PQP_REAL R1[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, T1[3] = {0, 0, 0}, R2[3][3];
        for (int i = 0; i < 9; i++) R2[i / 3][i % 3] = Rv[i];
        PQP_ToleranceResult tr;
        if (C2A_Tolerance(&tr, R1, T1, models[ab[0]], R2, T2, models[ab[1]], tol, 2) != 0) return 5;
        std::printf("%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d %d\n", tr.CloserThanTolerance(), tr.Distance(),
                    tr.P1()[0], tr.P1()[1], tr.P1()[2], tr.P2()[0], tr.P2()[1], tr.P2()[2], tr.NumBVTests(),
                    tr.NumTriTests());
        PQP_CollideResult cr;
        if (C2A_Collide(&cr, R1, T1, models[ab[0]], R2, T2, models[ab[1]], C2A_ALL_CONTACTS) != 0) return 6;
        std::printf("%d %d %d", cr.NumPairs(), cr.NumBVTests(), cr.NumTriTests());
        for (int i = 0; i < cr.NumPairs(); i++) std::printf(" %d %d", cr.Id1(i), cr.Id2(i));
        std::printf("\n");
        C2A_DistanceResult dr;
        if (C2A_Distance(&dr, R1, T1, models[ab[0]], R2, T2, models[ab[1]], 0.0, 0.0) != 0) return 7;
        std::printf("%.17g %d %d\n", dr.Distance(), dr.t1, dr.t2);
    }
    for (C2A_Model *o : models) delete o;
    return 0;
}
