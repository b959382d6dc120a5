/*
 * c2a_api.cpp -- the C++ drop-in API of include/c2a_gb300_cpp.h on top of the
 * C ABI.  Each entry point packs its arguments into c2a_query records, runs
 * them on the GPU and unpacks the results into the reference's structures.
 */
#include "../../../include/c2a_gb300_cpp.h"

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../common/c2a_motion.h"

namespace {

std::mutex g_mu;
c2a_context *g_ctx = nullptr;
int g_device = 0;

void pose_of(const Transform &t, double *out12)
{
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) out12[3 * i + j] = t.Rotation()[i][j];
        out12[9 + i] = t.Translation()[i];
    }
}

void set_transform(Transform &t, const double *R9, const double *T3)
{
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) t.Rotation()[i][j] = R9[3 * i + j];
        t.Translation()[i] = T3[i];
    }
}

int tri_index(const C2A_Model *m, const Tri *t, int fallback)
{
    if (!m || !t || m->tris.empty()) return fallback;
    const C2A_Tri *base = m->tris.data();
    const ptrdiff_t i = static_cast<const C2A_Tri *>(t) - base;
    return (i >= 0 && i < (ptrdiff_t)m->tris.size()) ? (int)i : fallback;
}

/* contacts arrive in visiting order; the reference's list is push_front */
void push_contacts(ContactFList &l, const c2a_contact *c, int n)
{
    for (int k = 0; k < n; k++)
        l.push_front(ContactF(c[k].type_a, c[k].type_b, c[k].fid_a, c[k].fid_b, c[k].tri_a, c[k].tri_b, c[k].pa,
                              c[k].pb, c[k].distance));
}

void fill_result(C2A_TimeOfContactResult &r, const c2a_result &g, C2A_Model *o1, C2A_Model *o2)
{
    r.num_bv_tests = (int)g.num_bv_tests;
    r.num_tri_tests = (int)g.num_tri_tests;
    r.distance = g.distance;
    r.mint = g.mint;
    r.toc = g.toc;
    r.collisionfree = g.collisionfree != 0;
    r.numCA = g.numCA;
    r.num_contact = g.num_contact;
    r.status = g.status;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) r.R_toc[i][j] = g.R_toc[0][3 * i + j];
        r.T_toc[i] = g.T_toc[0][i];
    }
    if (o1 && g.seed_a >= 0 && g.seed_a < o1->num_tris) r.last_triA = &o1->tris[g.seed_a];
    if (o2 && g.seed_b >= 0 && g.seed_b < o2->num_tris) r.last_triB = &o2->tris[g.seed_b];
}

/* contacts at a TOC pose when the solve's buffer was too small */
int exact_contacts(c2a_context *ctx, const c2a_query &q, double threshold, std::vector<c2a_contact> &out)
{
    c2a_result r;
    std::memset(&r, 0, sizeof(r));
    int cap = 1024;
    for (;;) {
        out.assign((size_t)cap, c2a_contact());
        if (c2a_contact_only_batch(ctx, &q, 1, &threshold, cap, &r, out.data()) != C2A_OK) return -1;
        if (r.num_contact <= cap) {
            out.resize((size_t)r.num_contact);
            return r.num_contact;
        }
        cap = r.num_contact;
    }
}

} // namespace

/* ------------------------------------------------------- LinearMath subset */
void Matrix3x3::Get_Value(Real v[3][3]) const
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v[i][j] = val[3 * i + j];
}
void Matrix3x3::Set_Value(const Real v[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) val[3 * i + j] = v[i][j];
}
void Matrix3x3::Set_Value(const Quaternion &q)
{
    const double qq[4] = {q.X(), q.Y(), q.Z(), q.W()};
    c2a::quat_to_mat(val, qq);
}

/* ------------------------------------------------------------- context */
int C2A_SetDevice(int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_ctx) return g_device == device ? 0 : C2A_ERR_INVALID_ARGUMENT;
    g_device = device;
    return 0;
}

c2a_context *C2A_DefaultContext()
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ctx) {
        c2a_status s = c2a_create(g_device, &g_ctx);
        if (s != C2A_OK) {
            fprintf(stderr, "c2a_gb300: cannot create the GPU context: %s\n", c2a_status_str(s));
            g_ctx = nullptr;
        }
    }
    return g_ctx;
}

/* ---------------------------------------------------------------- model */
C2A_Model::C2A_Model()
    : build_state(0), num_tris(0), last_tri(nullptr), num_bvs(0), maxdeep(0), ctx(nullptr), model_id(-1)
{
}

C2A_Model::~C2A_Model()
{
    if (ctx && model_id >= 0) c2a_model_free(ctx, model_id);
}

int C2A_Model::BeginModel(int n)
{
    const bool was_used = build_state != 0;
    if (ctx && model_id >= 0) c2a_model_free(ctx, model_id);
    model_id = -1;
    trisConst.clear();
    tris.clear();
    trisConst.reserve(n > 0 ? (size_t)n : 8);
    num_tris = 0;
    num_bvs = 0;
    last_tri = nullptr;
    build_state = 1;
    return was_used ? -4 /* PQP_ERR_BUILD_OUT_OF_SEQUENCE, C2A_PQP.cpp:109-117 */ : 0;
}

int C2A_Model::AddTri(const PQP_REAL *p1, const PQP_REAL *p2, const PQP_REAL *p3, int i, int i1, int i2, int i3)
{
    if (build_state == 0) BeginModel();
    else if (build_state == 2) return -4;
    C2A_Tri t;
    std::memcpy(t.p1, p1, sizeof(t.p1));
    std::memcpy(t.p2, p2, sizeof(t.p2));
    std::memcpy(t.p3, p3, sizeof(t.p3));
    t.id = i;
    t.index_[0] = i1;
    t.index_[1] = i2;
    t.index_[2] = i3;
    trisConst.push_back(t);
    num_tris = (int)trisConst.size();
    return 0;
}

int C2A_Model::AddTri(const PQP_REAL *p1, const PQP_REAL *p2, const PQP_REAL *p3, int id)
{
    return AddTri(p1, p2, p3, id, -1, -1, -1);
}

int C2A_Model::EndModel()
{
    if (build_state == 2) return -4;
    if (trisConst.empty()) return -5; /* PQP_ERR_BUILD_EMPTY_MODEL */
    ctx = C2A_DefaultContext();
    if (!ctx) return -1;
    const size_t n = trisConst.size();
    std::vector<double> v(9 * n);
    std::vector<int32_t> ids(n), vidx(3 * n);
    for (size_t i = 0; i < n; i++) {
        std::memcpy(&v[9 * i], trisConst[i].p1, 3 * sizeof(double));
        std::memcpy(&v[9 * i + 3], trisConst[i].p2, 3 * sizeof(double));
        std::memcpy(&v[9 * i + 6], trisConst[i].p3, 3 * sizeof(double));
        ids[i] = trisConst[i].id;
        for (int k = 0; k < 3; k++) vidx[3 * i + k] = trisConst[i].index_[k];
    }
    c2a_status s = c2a_model_build(ctx, (int32_t)n, v.data(), ids.data(), vidx.data(), &model_id);
    if (s != C2A_OK) return -(int)s;
    int32_t nt = 0, nn = 0, depth = 0;
    c2a_model_info(ctx, model_id, &nt, &nn, &depth);
    c2a_model_download(ctx, model_id, nullptr, nullptr, v.data(), ids.data(), vidx.data());
    tris.resize(n);
    for (size_t i = 0; i < n; i++) {
        std::memcpy(tris[i].p1, &v[9 * i], 3 * sizeof(double));
        std::memcpy(tris[i].p2, &v[9 * i + 3], 3 * sizeof(double));
        std::memcpy(tris[i].p3, &v[9 * i + 6], 3 * sizeof(double));
        tris[i].id = ids[i];
        for (int k = 0; k < 3; k++) tris[i].index_[k] = vidx[3 * i + k];
    }
    num_bvs = nn;
    maxdeep = depth;
    last_tri = &tris[0]; /* C2A_PQP.cpp:401 */
    build_state = 2;
    return 0;
}

/* ---------------------------------------------------------------- motion */
CInterpMotion::CInterpMotion() : m_toc_delta(1e-4), m_itpMode(GMP_IM_LINEAR), m_angVel(0), m_time(0) {}
CInterpMotion::~CInterpMotion() {}

bool CInterpMotion::integrate(const double dt, PQP_REAL R[3][3], PQP_REAL T[3])
{
    PQP_REAL qua[7];
    integrate(dt, qua);
    transform.Rotation().Get_Value(R);
    for (int i = 0; i < 3; i++) T[i] = transform.Translation()[i];
    return true;
}

CInterpMotion_Linear::CInterpMotion_Linear(const PQP_REAL R0[3][3], const PQP_REAL T0[3], const PQP_REAL R1[3][3],
                                           const PQP_REAL T1[3])
{
    double r0[9], r1[9], out[11];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            r0[3 * i + j] = R0[i][j];
            r1[3 * i + j] = R1[i][j];
        }
    set_transform(transform_s, r0, T0);
    set_transform(transform_t, r1, T1);
    transform = transform_s;
    c2a_motion_setup(r0, T0, r1, T1, out);
    m_axis.Set_Value(out[0], out[1], out[2]);
    m_angVel = out[3];
    cv.Set_Value(out[4], out[5], out[6]);
    m_time = 0;
}

CInterpMotion_Linear::~CInterpMotion_Linear() {}

bool CInterpMotion_Linear::integrate(const double dt, PQP_REAL qua[7])
{
    double p0[12], p1[12], R[9], T[3];
    pose_of(transform_s, p0);
    pose_of(transform_t, p1);
    c2a_motion_integrate(p0, p0 + 9, p1, p1 + 9, dt, R, T, qua);
    set_transform(transform, R, T);
    m_time = dt > 1 ? 1 : dt;
    return true;
}

/* --------------------------------------------------------------- results */
ContactF::ContactF(int ta, int tb, const int fa[3], const int fb[3], int tria, int trib, const PQP_REAL pa[3],
                   const PQP_REAL pb[3], PQP_REAL d)
    : FeatureType_A(ta), FeatureType_B(tb), TriangleID_A(tria), TriangleID_B(trib), Distance(d)
{
    for (int i = 0; i < 3; i++) {
        FeatureID_A[i] = fa[i];
        FeatureID_B[i] = fb[i];
        P_A[i] = pa[i];
        P_B[i] = pb[i];
    }
}

C2A_TimeOfContactResult::C2A_TimeOfContactResult()
    : num_bv_tests(0), num_tri_tests(0), query_time_secs(0), rel_err(0), abs_err(0), UpboundTOC(1), distance(0),
      qsize(2), mint(1), toc(0), collisionfree(true), numCA(0), num_contact(0), last_triA(nullptr),
      last_triB(nullptr), status(0)
{
    std::memset(R, 0, sizeof(R));
    std::memset(T, 0, sizeof(T));
    std::memset(p1, 0, sizeof(p1));
    std::memset(p2, 0, sizeof(p2));
    std::memset(R_toc, 0, sizeof(R_toc));
    std::memset(T_toc, 0, sizeof(T_toc));
}

/* ------------------------------------------------------------------ API */
static void make_query(c2a_query &q, const Transform &a0, const Transform &a1, const C2A_Model *o1, const Transform &b0,
                       const Transform &b1, const C2A_Model *o2, int seed_a, int seed_b)
{
    std::memset(&q, 0, sizeof(q));
    q.model_a = o1 ? o1->model_id : -1;
    q.model_b = o2 ? o2->model_id : -1;
    q.seed_a = seed_a;
    q.seed_b = seed_b;
    pose_of(a0, q.pose);
    pose_of(a1, q.pose + 12);
    pose_of(b0, q.pose + 24);
    pose_of(b1, q.pose + 36);
}

static c2a_params make_params(double tol_d, double tol_t, double toc_delta, int with_contacts, int slots)
{
    c2a_params p;
    std::memset(&p, 0, sizeof(p));
    p.tol_d = tol_d;
    p.tol_t = tol_t;
    p.toc_delta = toc_delta;
    p.contact_abs = 0.001;
    p.with_contacts = with_contacts;
    p.max_iters = 150;
    p.qsize = 64;
    p.contacts_per_query = slots;
    return p;
}

PQP_REAL C2A_QueryTimeOfContact(CInterpMotion *m1, CInterpMotion *m2, C2A_TimeOfContactResult *res, C2A_Model *o1,
                                C2A_Model *o2, PQP_REAL tolerance_d, PQP_REAL tolerance_t, int qsize)
{
    c2a_context *ctx = o1 ? o1->ctx : nullptr;
    if (!ctx || !m1 || !m2 || !res || !o2) return 0;
    c2a_query q;
    make_query(q, m1->transform_s, m1->transform_t, o1, m2->transform_s, m2->transform_t, o2,
               tri_index(o1, res->last_triA, 0), tri_index(o2, res->last_triB, 0));
    c2a_params p = make_params(tolerance_d, tolerance_t, m1->m_toc_delta, 0, 0);
    p.qsize = qsize;
    c2a_result r;
    std::memset(&r, 0, sizeof(r));
    if (c2a_solve_batch(ctx, &q, 1, &p, &r, nullptr) != C2A_OK && r.status == 0) r.status = C2A_QUERY_BAD_INPUT;
    fill_result(*res, r, o1, o2);
    res->num_contact = 0;
    res->UpboundTOC = 1;
    if (!res->collisionfree) {
        PQP_REAL qua[7];
        m1->integrate(res->toc, qua); /* like the reference: objmotion1 ends at the TOC */
    }
    return res->toc;
}

int C2A_TimeOfContactStep(CInterpMotion *m1, CInterpMotion *m2, C2A_TimeOfContactResult *res, PQP_REAL R1[3][3],
                          PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3], PQP_REAL T2[3], C2A_Model *o2,
                          PQP_REAL tolerance_t, PQP_REAL tolerance_d)
{
    c2a_context *ctx = o1 ? o1->ctx : nullptr;
    if (!ctx || !m1 || !m2 || !res || !o2) return -1;
    c2a_query q;
    make_query(q, m1->transform_s, m1->transform_t, o1, m2->transform_s, m2->transform_t, o2,
               tri_index(o1, res->last_triA, 0), tri_index(o2, res->last_triB, 0));
    const double lambda = m1->m_time;
    const int32_t num_ca = res->numCA;
    const double prev_mint = res->mint;
    c2a_params p = make_params(tolerance_d, tolerance_t, m1->m_toc_delta, 0, 0);
    c2a_result r;
    std::memset(&r, 0, sizeof(r));
    c2a_status s = c2a_toc_step_batch(ctx, &q, 1, &lambda, &num_ca, &prev_mint, &p, &r);
    res->distance = r.distance;
    res->mint = r.mint;
    res->num_bv_tests += (int)r.num_bv_tests;
    res->num_tri_tests += (int)r.num_tri_tests;
    res->status = r.status;
    res->UpboundTOC = 1.0 - lambda;
    if (o1 && r.seed_a >= 0 && r.seed_a < o1->num_tris) res->last_triA = &o1->tris[r.seed_a];
    if (o2 && r.seed_b >= 0 && r.seed_b < o2->num_tris) res->last_triB = &o2->tris[r.seed_b];
    /* model-level relative transform, as the reference leaves it in res */
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) res->R[i][j] = R1[0][i] * R2[0][j] + R1[1][i] * R2[1][j] + R1[2][i] * R2[2][j];
        const double d0 = T2[0] - T1[0], d1 = T2[1] - T1[1], d2 = T2[2] - T1[2];
        res->T[i] = R1[0][i] * d0 + R1[1][i] * d1 + R1[2][i] * d2;
    }
    return s == C2A_OK ? 0 : -1;
}

static PQP_REAL contact_query(C2A_TimeOfContactResult *res, const Transform &a, C2A_Model *o1, const Transform &b,
                              C2A_Model *o2, double threshold)
{
    c2a_context *ctx = o1 ? o1->ctx : nullptr;
    if (!ctx || !res || !o2) return 0;
    c2a_query q;
    make_query(q, a, a, o1, b, b, o2, 0, 0);
    std::vector<c2a_contact> c;
    const int n = exact_contacts(ctx, q, threshold, c);
    if (n < 0) {
        res->status |= C2A_QUERY_BAD_INPUT;
        return 0;
    }
    res->num_contact = n;
    push_contacts(res->cont_l, c.data(), n);
    return 0;
}

PQP_REAL C2A_QueryContact(CInterpMotion *m1, CInterpMotion *m2, C2A_TimeOfContactResult *res, C2A_Model *o1,
                          C2A_Model *o2, double threshold)
{
    if (!m1 || !m2 || !res) return 0;
    res->num_contact = 0;
    res->UpboundTOC = 1;
    return contact_query(res, m1->transform, o1, m2->transform, o2, threshold);
}

PQP_REAL C2A_QueryContactOnly(C2A_TimeOfContactResult *res, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1,
                              PQP_REAL R2[3][3], PQP_REAL T2[3], C2A_Model *o2, double threshold)
{
    if (!res) return 0;
    res->cont_l.clear();
    res->num_contact = 0;
    res->UpboundTOC = 1;
    double a[12], b[12];
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            a[3 * i + j] = R1[i][j];
            b[3 * i + j] = R2[i][j];
        }
        a[9 + i] = T1[i];
        b[9 + i] = T2[i];
    }
    Transform ta, tb;
    set_transform(ta, a, a + 9);
    set_transform(tb, b, b + 9);
    return contact_query(res, ta, o1, tb, o2, threshold);
}

int C2A_SolveBatch(const C2A_BatchQuery *queries, int n, PQP_REAL th_ca, C2A_TimeOfContactResult *results,
                   int contacts_per_query)
{
    if (n <= 0) return 0;
    if (!queries || !results || !queries[0].obj1 || !queries[0].obj1->ctx) return n;
    c2a_context *ctx = queries[0].obj1->ctx;
    std::vector<c2a_query> q((size_t)n);
    for (int i = 0; i < n; i++) {
        const C2A_BatchQuery &b = queries[i];
        const int sa = b.seed1 >= 0 ? b.seed1 : tri_index(b.obj1, b.obj1 ? b.obj1->last_tri : nullptr, 0);
        const int sb = b.seed2 >= 0 ? b.seed2 : tri_index(b.obj2, b.obj2 ? b.obj2->last_tri : nullptr, 0);
        make_query(q[i], *b.trans00, *b.trans01, b.obj1, *b.trans10, *b.trans11, b.obj2, sa, sb);
    }
    const double tol = th_ca > 0 ? th_ca : 1e-4; /* C2A_Solve's constants when th_ca is not given */
    c2a_params p = make_params(tol, 1e-4, tol, 1, contacts_per_query);
    std::vector<c2a_result> r((size_t)n);
    std::vector<c2a_contact> c((size_t)n * (size_t)contacts_per_query);
    c2a_solve_batch(ctx, q.data(), n, &p, r.data(), contacts_per_query ? c.data() : nullptr);
    int failed = 0;
    for (int i = 0; i < n; i++) {
        C2A_TimeOfContactResult &res = results[i];
        res.cont_l.clear();
        fill_result(res, r[i], queries[i].obj1, queries[i].obj2);
        if (!res.collisionfree) {
            if (r[i].num_contact <= contacts_per_query) {
                push_contacts(res.cont_l, c.data() + r[i].contact_offset, r[i].num_contact);
            } else {
                c2a_query qt = q[i];
                std::memcpy(qt.pose, r[i].R_toc[0], 9 * sizeof(double));
                std::memcpy(qt.pose + 9, r[i].T_toc[0], 3 * sizeof(double));
                std::memcpy(qt.pose + 24, r[i].R_toc[1], 9 * sizeof(double));
                std::memcpy(qt.pose + 33, r[i].T_toc[1], 3 * sizeof(double));
                std::vector<c2a_contact> all;
                const int k = exact_contacts(ctx, qt, 2 * r[i].distance + p.contact_abs, all);
                if (k >= 0) push_contacts(res.cont_l, all.data(), k);
                res.status &= ~C2A_QUERY_CONTACT_OVERFLOW;
            }
        }
        if (res.status & ~C2A_QUERY_ITER_CAP & ~C2A_QUERY_CONTACT_OVERFLOW) failed++;
    }
    return failed;
}

C2A_Result C2A_Solve(Transform *trans00, Transform *trans01, C2A_Model *obj1, Transform *trans10, Transform *trans11,
                     C2A_Model *obj2, Transform &trans0, Transform &trans1, PQP_REAL &time_of_contact,
                     int &number_of_iteration, int &number_of_contact, PQP_REAL th_ca, C2A_TimeOfContactResult &dres)
{
    C2A_BatchQuery b;
    b.trans00 = trans00;
    b.trans01 = trans01;
    b.obj1 = obj1;
    b.trans10 = trans10;
    b.trans11 = trans11;
    b.obj2 = obj2;
    b.seed1 = tri_index(obj1, dres.last_triA, -1);
    b.seed2 = tri_index(obj2, dres.last_triB, -1);
    C2A_SolveBatch(&b, 1, th_ca, &dres, 256);
    if (!dres.collisionfree) {
        dres.mint = 1; /* the contact query resets it (C2A.cpp:1757) */
        /* the TOC poses come back with the result (C2A.cpp:2411-2431) */
        const double pa[12] = {dres.R_toc[0][0], dres.R_toc[0][1], dres.R_toc[0][2], dres.R_toc[1][0],
                               dres.R_toc[1][1], dres.R_toc[1][2], dres.R_toc[2][0], dres.R_toc[2][1],
                               dres.R_toc[2][2], dres.T_toc[0], dres.T_toc[1], dres.T_toc[2]};
        set_transform(trans0, pa, pa + 9);
        double p0[12], p1[12], R[9], T[3], qua[7];
        pose_of(*trans10, p0);
        pose_of(*trans11, p1);
        c2a_motion_integrate(p0, p0 + 9, p1, p1 + 9, dres.toc, R, T, qua);
        set_transform(trans1, R, T);
    }
    time_of_contact = dres.toc;
    number_of_contact = dres.num_contact;
    number_of_iteration = dres.numCA;
    return TOCFound;
}

/* ----------------------------------------------- static proximity queries */
namespace {
/* model a placed by (R1, T1), model b by (R2, T2); seeds from the models' last_tri */
c2a_query static_query(const PQP_REAL R1[3][3], const PQP_REAL T1[3], const C2A_Model *o1, const PQP_REAL R2[3][3],
                       const PQP_REAL T2[3], const C2A_Model *o2)
{
    c2a_query q;
    std::memset(&q, 0, sizeof(q));
    q.model_a = o1 ? o1->model_id : -1;
    q.model_b = o2 ? o2->model_id : -1;
    q.seed_a = tri_index(o1, o1 ? o1->last_tri : nullptr, 0);
    q.seed_b = tri_index(o2, o2 ? o2->last_tri : nullptr, 0);
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            q.pose[3 * i + j] = R1[i][j];
            q.pose[24 + 3 * i + j] = R2[i][j];
        }
        q.pose[9 + i] = T1[i];
        q.pose[33 + i] = T2[i];
    }
    return q;
}

/* the result's R, T: model 2 in model 1's frame (MTxM, VmV, MTxV) */
void relative(const PQP_REAL R1[3][3], const PQP_REAL T1[3], const PQP_REAL R2[3][3], const PQP_REAL T2[3],
              PQP_REAL R[3][3], PQP_REAL T[3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) R[i][j] = R1[0][i] * R2[0][j] + R1[1][i] * R2[1][j] + R1[2][i] * R2[2][j];
    const PQP_REAL d[3] = {T2[0] - T1[0], T2[1] - T1[1], T2[2] - T1[2]};
    for (int i = 0; i < 3; i++) T[i] = R1[0][i] * d[0] + R1[1][i] * d[1] + R1[2][i] * d[2];
}
} // namespace

int C2A_Distance(C2A_DistanceResult *result, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                 PQP_REAL T2[3], C2A_Model *o2, PQP_REAL rel_err, PQP_REAL abs_err, int qsize)
{
    if (!result || !o1 || !o2 || rel_err != 0 || abs_err != 0) return C2A_ERR_INVALID_ARGUMENT;
    const c2a_query q = static_query(R1, T1, o1, R2, T2, o2);
    c2a_distance_result r;
    const c2a_status st = c2a_distance_batch(o1->ctx, &q, 1, &r);
    if (st) return st;
    relative(R1, T1, R2, T2, result->R, result->T);
    result->rel_err = rel_err;
    result->abs_err = abs_err;
    result->qsize = qsize;
    result->distance = r.distance;
    std::memcpy(result->p1, r.p1, sizeof(result->p1));
    std::memcpy(result->p2, r.p2, sizeof(result->p2));
    result->last_triA = o1->GetTriangle(r.tri_a);
    result->last_triB = o2->GetTriangle(r.tri_b);
    result->t1 = result->last_triA->id;
    result->t2 = result->last_triB->id;
    result->num_bv_tests = result->num_tri_tests = 0; /* the batch query reports no counters */
    return C2A_OK;
}

int C2A_Tolerance(PQP_ToleranceResult *res, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                  PQP_REAL T2[3], C2A_Model *o2, PQP_REAL tolerance, int qsize)
{
    (void)qsize; /* the qsize-2 order (the reference's default and the demo's) */
    if (!res || !o1 || !o2) return C2A_ERR_INVALID_ARGUMENT;
    const c2a_query q = static_query(R1, T1, o1, R2, T2, o2);
    c2a_tolerance_result r;
    const double tol = tolerance;
    const c2a_status st = c2a_tolerance_batch(o1->ctx, &q, 1, &tol, &r);
    if (st) return st;
    relative(R1, T1, R2, T2, res->R, res->T);
    res->tolerance = tolerance < 0 ? 0 : tolerance;
    res->closer_than_tolerance = r.closer;
    res->distance = r.closer ? r.distance : 0.0;
    std::memcpy(res->p1, r.p1, sizeof(res->p1));
    std::memcpy(res->p2, r.p2, sizeof(res->p2));
    res->num_bv_tests = (int)r.num_bv_tests;
    res->num_tri_tests = (int)r.num_tri_tests;
    return C2A_OK;
}

int C2A_Collide(PQP_CollideResult *result, PQP_REAL R1[3][3], PQP_REAL T1[3], C2A_Model *o1, PQP_REAL R2[3][3],
                PQP_REAL T2[3], C2A_Model *o2, int flag)
{
    if (!result || !o1 || !o2) return C2A_ERR_INVALID_ARGUMENT;
    const c2a_query q = static_query(R1, T1, o1, R2, T2, o2);
    c2a_collide_result r;
    int slots = 1024;
    std::vector<int32_t> pairs;
    for (;;) { /* a second launch with room for every pair when the first overflowed */
        pairs.assign(2 * (size_t)slots, 0);
        const c2a_status st = c2a_collide_batch(o1->ctx, &q, 1, flag, slots, &r, pairs.data());
        if (st) return st;
        if (r.num_pairs <= slots) break;
        slots = r.num_pairs;
    }
    relative(R1, T1, R2, T2, result->R, result->T);
    result->pairs.resize((size_t)r.num_pairs);
    for (int k = 0; k < r.num_pairs; k++) result->pairs[(size_t)k] = CollisionPair{pairs[2 * k], pairs[2 * k + 1]};
    result->num_bv_tests = (int)r.num_bv_tests;
    result->num_tri_tests = (int)r.num_tri_tests;
    return C2A_OK;
}
