// Exercises the C++ drop-in API the way the reference's demo does
// (CCDDemo/mainTorusknot.cpp:445-540 builds models with AddTri/EndModel,
// :308-325 calls C2A_Solve with dres.last_triA/B set): reads a mesh and
// queries from a binary file, prints one line per query for C2A_Solve and
// then for C2A_SolveBatch: toc numCA num_contact collisionfree.
#include <cstdio>
#include <vector>

#include "c2a_gb300_cpp.h"

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    if (std::fread(hdr, sizeof(int), 3, f) != 3) return 2;
    const int nt = hdr[0], nv = hdr[1], nq = hdr[2];
    std::vector<double> v(3 * (size_t)nv), poses(48 * (size_t)nq);
    std::vector<int> faces(3 * (size_t)nt);
    double th_ca = 0;
    if (std::fread(v.data(), sizeof(double), v.size(), f) != v.size() ||
        std::fread(faces.data(), sizeof(int), faces.size(), f) != faces.size() ||
        std::fread(poses.data(), sizeof(double), poses.size(), f) != poses.size() ||
        std::fread(&th_ca, sizeof(double), 1, f) != 1)
        return 2;
    std::fclose(f);

    C2A_Model model;
    model.BeginModel();
    for (int i = 0; i < nt; i++) {
        const int a = faces[3 * i], b = faces[3 * i + 1], c = faces[3 * i + 2];
        model.AddTri(&v[3 * a], &v[3 * b], &v[3 * c], i, a, b, c);
    }
    if (model.EndModel() != 0) return 3;

    std::vector<Transform> tf(4 * (size_t)nq);
    for (int q = 0; q < nq; q++)
        for (int k = 0; k < 4; k++) {
            const double *p = &poses[48 * (size_t)q + 12 * k];
            Transform &t = tf[4 * (size_t)q + k];
            for (int i = 0; i < 3; i++) {
                for (int j = 0; j < 3; j++) t.Rotation()[i][j] = p[3 * i + j];
                t.Translation()[i] = p[9 + i];
            }
        }

    for (int q = 0; q < nq; q++) {
        C2A_TimeOfContactResult dres;
        dres.last_triA = model.last_tri;
        dres.last_triB = model.last_tri;
        Transform t0, t1;
        PQP_REAL toc = 0;
        int iters = 0, ncont = 0;
        C2A_Solve(&tf[4 * q], &tf[4 * q + 1], &model, &tf[4 * q + 2], &tf[4 * q + 3], &model, t0, t1, toc, iters,
                  ncont, th_ca, dres);
        std::printf("%.17g %d %d %d\n", toc, iters, ncont, dres.collisionfree ? 1 : 0);
    }

    std::vector<C2A_BatchQuery> bq((size_t)nq);
    for (int q = 0; q < nq; q++) {
        C2A_BatchQuery &b = bq[q];
        b.trans00 = &tf[4 * q];
        b.trans01 = &tf[4 * q + 1];
        b.trans10 = &tf[4 * q + 2];
        b.trans11 = &tf[4 * q + 3];
        b.obj1 = b.obj2 = &model;
        b.seed1 = b.seed2 = -1;
    }
    std::vector<C2A_TimeOfContactResult> res((size_t)nq);
    if (C2A_SolveBatch(bq.data(), nq, th_ca, res.data()) != 0) return 4;
    for (int q = 0; q < nq; q++)
        std::printf("%.17g %d %d %d\n", res[q].toc, res[q].numCA, res[q].num_contact, res[q].collisionfree ? 1 : 0);
    return 0;
}
