/*
 * Test infrastructure only: a C-ABI wrapper around the reference NBodylib KDTree,
 * compiled from the reference's own unmodified sources (see oracle/Makefile) into
 * oracle/_ref/libnbref.so. The parity tests and the golden-fixture generator load it
 * through ctypes to run the reference itself on the same inputs as the GPU path.
 *
 * Every function builds on the reference's public API (src/KDTree/KDTree.h):
 *   KDTree(Particle*, N, b, TreeType, KernType, KernRes, ..., Period)  KDTree.h:229-245
 *   FindNearest / FindNearestPos(tt | x)                                KDTree.h:307-313
 *   CalcDensity, CalcVelDensity, CalcDensityParticle, CalcVelDensityParticle  KDTree.h:407-425
 *   FOF, FOFCriterion                                                   KDTree.h:480-503
 *   SearchBallPos(tt), SearchBallPosTagged(tt | x)                      KDTree.h:342-373
 * Results are returned in input order (the reference's particle ID = input index,
 * src/KDTree/KDTree.cxx:1291), and neighbour lists hold IDs, not tree indices.
 */
#include <KDTree.h>
#include <vector>
#include <cstring>
#include <algorithm>
#include <chrono>
#ifdef USEOPENMP
#include <omp.h>
#endif

using namespace NBody;

namespace {
struct RefTree {
    std::vector<Particle> parts;   // permuted in place by the reference constructor
    std::vector<int> tree_of_id;   // ID -> tree index
    KDTree* tree = nullptr;
    int n = 0;
    double period[3] = {0, 0, 0};
    bool periodic = false;
    double build_seconds = 0;
};

void refresh_index(RefTree* r) {
    r->tree_of_id.assign(r->n, -1);
    for (int t = 0; t < r->n; t++) r->tree_of_id[r->parts[t].GetID()] = t;
}
}  // namespace

extern "C" {

/* The constructor with its Aniso argument (KDTree.h:229-245): -1 plain phase-space
   distance, 0 local metric (the default) for phase-space trees. */
void* ref_create_ex(const double* pos, const double* vel, const double* mass, int n, int b,
                    int treetype, int kerntype, int kernres, const double* period, int nthreads,
                    int aniso);

void* ref_create(const double* pos, const double* vel, const double* mass, int n, int b,
                 int treetype, int kerntype, int kernres, const double* period, int nthreads) {
    return ref_create_ex(pos, vel, mass, n, b, treetype, kerntype, kernres, period, nthreads, 0);
}

void* ref_create_ex(const double* pos, const double* vel, const double* mass, int n, int b,
                    int treetype, int kerntype, int kernres, const double* period, int nthreads,
                    int aniso) {
#ifdef USEOPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    RefTree* r = new RefTree;
    r->n = n;
    r->parts.resize(n);
    for (int i = 0; i < n; i++) {
        Particle& p = r->parts[i];
        p.SetMass(mass ? mass[i] : 1.0);
        p.SetPosition(pos[3 * i + 0], pos[3 * i + 1], pos[3 * i + 2]);
        if (vel) p.SetVelocity(vel[3 * i + 0], vel[3 * i + 1], vel[3 * i + 2]);
        else p.SetVelocity(0.0, 0.0, 0.0);
        p.SetID(i);
        p.SetPID(i);
    }
    double per[3];
    double* pp = nullptr;
    if (period) {
        for (int k = 0; k < 3; k++) per[k] = period[k];
        pp = per;
        r->periodic = true;
        for (int k = 0; k < 3; k++) r->period[k] = period[k];
    }
    auto t0 = std::chrono::steady_clock::now();
    r->tree = new KDTree(r->parts.data(), n, b, treetype, kerntype, kernres, 0, aniso, 0, pp);
    auto t1 = std::chrono::steady_clock::now();
    r->build_seconds = std::chrono::duration<double>(t1 - t0).count();
    refresh_index(r);
    return r;
}

double ref_build_seconds(void* h) { return ((RefTree*)h)->build_seconds; }

void ref_destroy(void* h) {
    RefTree* r = (RefTree*)h;
    delete r->tree;
    delete r;
}

int ref_num_nodes(void* h) { return ((RefTree*)h)->tree->GetNumNodes(); }
int ref_num_leaves(void* h) { return ((RefTree*)h)->tree->GetNumLeafNodes(); }
double ref_kernnorm(void* h) { return ((RefTree*)h)->tree->GetKernNorm(); }

void ref_ids(void* h, int* ids) {
    RefTree* r = (RefTree*)h;
    for (int t = 0; t < r->n; t++) ids[t] = r->parts[t].GetID();
}

/* Leaf membership: for each tree index, the start of its leaf (walks the node tree). */
static void walk_leaves(Node* node, int* leaf_start) {
    if (node->GetLeaf()) {
        for (int i = node->GetStart(); i < node->GetEnd(); i++) leaf_start[i] = node->GetStart();
        return;
    }
    walk_leaves(((SplitNode*)node)->GetLeft(), leaf_start);
    walk_leaves(((SplitNode*)node)->GetRight(), leaf_start);
}
void ref_leaf_start(void* h, int* leaf_start_by_tree_index) {
    RefTree* r = (RefTree*)h;
    walk_leaves(r->tree->GetRoot(), leaf_start_by_tree_index);
}

/* method 0: FindNearest(tt), 1: FindNearestPos(tt). Row i is the query with ID i. */
int ref_knn(void* h, int method, int k, int nthreads, int* nn_ids, double* d2) {
    RefTree* r = (RefTree*)h;
    int n = r->n;
#ifdef USEOPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        std::vector<int> nn(k);
        std::vector<double> dd(k);
#ifdef USEOPENMP
#pragma omp for schedule(guided)
#endif
        for (int id = 0; id < n; id++) {
            int t = r->tree_of_id[id];
            if (method == 0) r->tree->FindNearest(t, nn.data(), dd.data(), k);
            else r->tree->FindNearestPos(t, nn.data(), dd.data(), k);
            for (int j = 0; j < k; j++) {
                nn_ids[(size_t)id * k + j] = nn[j] >= 0 ? r->parts[nn[j]].GetID() : -1;
                d2[(size_t)id * k + j] = dd[j];
            }
        }
    }
    return 0;
}

/* FindNearestPos(x) for nq coordinates (row-major xyz). */
int ref_knn_pos(void* h, const double* x, int nq, int k, int* nn_ids, double* d2) {
    RefTree* r = (RefTree*)h;
    std::vector<int> nn(k);
    std::vector<double> dd(k);
    for (int q = 0; q < nq; q++) {
        double xx[3] = {x[3 * q], x[3 * q + 1], x[3 * q + 2]};
        r->tree->FindNearestPos(xx, nn.data(), dd.data(), k);
        for (int j = 0; j < k; j++) {
            nn_ids[(size_t)q * k + j] = nn[j] >= 0 ? r->parts[nn[j]].GetID() : -1;
            d2[(size_t)q * k + j] = dd[j];
        }
    }
    return 0;
}

/* FindNearest(Double_t* x) (KDFindNearest.cxx:460-507) for nq coordinates of the tree's
   space: nd = 3 (positions, or velocities for a velocity tree) or 6 (phase space). */
int ref_knn_coord(void* h, const double* x, int nq, int nd, int k, int* nn_ids, double* d2) {
    RefTree* r = (RefTree*)h;
    std::vector<int> nn(k);
    std::vector<double> dd(k);
    for (int q = 0; q < nq; q++) {
        double xx[6];
        for (int j = 0; j < nd; j++) xx[j] = x[(size_t)nd * q + j];
        r->tree->FindNearest(xx, nn.data(), dd.data(), k);
        for (int j = 0; j < k; j++) {
            nn_ids[(size_t)q * k + j] = nn[j] >= 0 ? r->parts[nn[j]].GetID() : -1;
            d2[(size_t)q * k + j] = dd[j];
        }
    }
    return 0;
}

int ref_density(void* h, int k, double* rho) {
    RefTree* r = (RefTree*)h;
    r->tree->CalcDensity(k);
    for (int t = 0; t < r->n; t++) rho[r->parts[t].GetID()] = r->parts[t].GetDensity();
    return 0;
}

int ref_veldensity(void* h, int nsmooth, int nsearch, double* out) {
    RefTree* r = (RefTree*)h;
    r->tree->CalcVelDensity(nsmooth, nsearch);
    for (int t = 0; t < r->n; t++) out[r->parts[t].GetID()] = r->parts[t].GetDensity();
    return 0;
}

double ref_density_particle(void* h, int id, int k) {
    RefTree* r = (RefTree*)h;
    return r->tree->CalcDensityParticle(r->tree_of_id[id], k);
}

double ref_veldensity_particle(void* h, int id, int nsmooth, int nsearch) {
    RefTree* r = (RefTree*)h;
    return r->tree->CalcVelDensityParticle(r->tree_of_id[id], nsmooth, nsearch);
}

double ref_density_position(void* h, const double* x, int k) {
    RefTree* r = (RefTree*)h;
    Double_t xq[3] = {x[0], x[1], x[2]};
    return r->tree->CalcDensityPosition(xq, k, (Double_t*)NULL);
}

double ref_veldensity_position(void* h, const double* x, const double* v, int nsmooth,
                               int nsearch) {
    RefTree* r = (RefTree*)h;
    Double_t xq[3] = {x[0], x[1], x[2]}, vq[3] = {v[0], v[1], v[2]};
    return r->tree->CalcVelDensityPosition(xq, vq, nsmooth, nsearch);
}

int ref_fof(void* h, double ll, int minnum, int order, int* group, int* ngroup) {
    RefTree* r = (RefTree*)h;
    Int_t ng = 0;
    Int_t* g = r->tree->FOF(ll, ng, minnum, order);
    std::memcpy(group, g, sizeof(int) * r->n);  // FOF's array is indexed by ID
    delete[] g;
    *ngroup = ng;
    return 0;
}

int ref_fof_criterion(void* h, int cmp, const double* params, int minnum, int order, int* group,
                      int* ngroup) {
    RefTree* r = (RefTree*)h;
    double p[20];
    for (int i = 0; i < 20; i++) p[i] = params[i];
    FOFcompfunc f = cmp == 0 ? FOF3d : (cmp == 1 ? FOFVel : FOF6d);
    Int_t ng = 0;
    Int_t* g = r->tree->FOFCriterion(f, p, ng, minnum, order);
    std::memcpy(group, g, sizeof(int) * r->n);
    delete[] g;
    *ngroup = ng;
    return 0;
}

/* SearchBallPosTagged(tt): returns the count; out_ids receives IDs (unsorted). */
int ref_ball_tagged(void* h, int id, double fdist2, int* out_ids) {
    RefTree* r = (RefTree*)h;
    std::vector<Int_t> v = r->tree->SearchBallPosTagged((Int_t)r->tree_of_id[id], fdist2);
    for (size_t i = 0; i < v.size(); i++) out_ids[i] = r->parts[v[i]].GetID();
    return (int)v.size();
}

int ref_ball_tagged_pos(void* h, const double* x, double fdist2, int* out_ids) {
    RefTree* r = (RefTree*)h;
    double xx[3] = {x[0], x[1], x[2]};
    std::vector<Int_t> v = r->tree->SearchBallPosTagged(xx, fdist2);
    for (size_t i = 0; i < v.size(); i++) out_ids[i] = r->parts[v[i]].GetID();
    return (int)v.size();
}

/* SearchBallPos(tt): ID-indexed marking arrays, as the reference writes them. */
int ref_ball_mark(void* h, int id, double fdist2, int imark, int* mark, double* dist2) {
    RefTree* r = (RefTree*)h;
    r->tree->SearchBallPos((Int_t)r->tree_of_id[id], fdist2, imark, mark, dist2);
    return 0;
}

// ---- FOFNNCriterion / FOFNNDistCriterion (KDFOF.cxx:380-640). nn rows by tree index.
// The distance form uses distfunc = the largest squared distance of the row.
static Double_t row_max(Int_t num, Double_t* d2) {
    Double_t m = d2[0];
    for (Int_t j = 1; j < num; j++) m = d2[j] > m ? d2[j] : m;
    return m;
}

int ref_fof_nn(void* h, int cmp, const double* params, int numnn, const int* nn,
               const double* dist2, int npc, const int* pidx, int minnum, int* group,
               int* ngroup) {
    RefTree* r = (RefTree*)h;
    double p[20];
    for (int i = 0; i < 20; i++) p[i] = params[i];
    FOFcompfunc f = cmp == 0 ? FOF3d : (cmp == 1 ? FOFVel : FOF6d);
    std::vector<Int_t*> rows(r->n);
    std::vector<Double_t*> drows(r->n);
    std::vector<Int_t> flat((size_t)r->n * numnn);
    std::vector<Double_t> dflat((size_t)r->n * numnn);
    for (int i = 0; i < r->n; i++) {
        rows[i] = &flat[(size_t)i * numnn];
        drows[i] = &dflat[(size_t)i * numnn];
        for (int j = 0; j < numnn; j++) {
            rows[i][j] = nn[(size_t)i * numnn + j];
            if (dist2) drows[i][j] = dist2[(size_t)i * numnn + j];
        }
    }
    std::vector<Int_t> npca(pidx ? pidx : (const int*)nullptr, pidx ? pidx + npc : nullptr);
    Int_t ng = 0;
    Int_t* g = dist2 ? r->tree->FOFNNDistCriterion(f, p, numnn, rows.data(), drows.data(), row_max,
                                                    npc, npca.data(), ng, minnum)
                     : r->tree->FOFNNCriterion(f, p, numnn, rows.data(), ng, minnum);
    std::memcpy(group, g, sizeof(int) * r->n);
    delete[] g;
    *ngroup = ng;
    return 0;
}

// ---- SPH smoothing (KDCalcSmoothQuantities.cxx:393-766, 922-1091, 1209-1306, 1539-1700).
// rho != NULL: set the particles' densities and pass densityset = 1; otherwise the
// reference computes CalcDensity(Nsmooth) itself (densityset = 0).
static int set_rho(RefTree* r, const double* rho) {
    if (!rho) return 0;
    for (int t = 0; t < r->n; t++) r->parts[t].SetDensity(rho[r->parts[t].GetID()]);
    return 1;
}

int ref_smooth_vel_moments(void* h, int which, int nsmooth, const double* rho,
                           const double* smvel, const double* disp, double* out) {
    RefTree* r = (RefTree*)h;
    int ds = set_rho(r, rho);
    int n = r->n;
    Coordinate* sv = nullptr;
    Matrix* dm = nullptr;
    if (which >= 1) {
        sv = new Coordinate[n];
        for (int i = 0; i < n; i++) sv[i] = Coordinate(smvel[3 * (size_t)i], smvel[3 * (size_t)i + 1], smvel[3 * (size_t)i + 2]);
    }
    if (which >= 2) {
        dm = new Matrix[n];
        for (int i = 0; i < n; i++) dm[i] = Matrix(&disp[9 * (size_t)i]);
    }
    if (which == 1) {
        Matrix* m = r->tree->CalcSmoothVelDisp(sv, nsmooth, ds, 1);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) out[9 * (size_t)i + 3 * k + l] = m[i](k, l);
        delete[] m;
    } else {
        Coordinate* c = which == 0 ? r->tree->CalcSmoothVel(nsmooth, ds)
                      : which == 2 ? r->tree->CalcSmoothVelSkew(sv, dm, nsmooth, ds, 1, 1)
                                   : r->tree->CalcSmoothVelKurtosis(sv, dm, nsmooth, ds, 1, 1);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) out[3 * (size_t)i + k] = c[i][k];
        delete[] c;
    }
    delete[] sv;
    delete[] dm;
    return 0;
}

int ref_veldensity_phys(void* h, int nsmooth, int nsearch, const double* rho, double* out) {
    RefTree* r = (RefTree*)h;
    int ds = set_rho(r, rho);
    Double_t* v = r->tree->CalcVelDensityWithPhysDensity(nsmooth, nsearch, ds);
    for (int i = 0; i < r->n; i++) out[i] = v[i];
    delete[] v;
    return 0;
}

double ref_veldensity_phys_particle(void* h, int id, int nsmooth, int nsearch, const double* rho) {
    RefTree* r = (RefTree*)h;
    int ds = set_rho(r, rho);
    return r->tree->CalcVelDensityWithPhysDensityParticle(r->tree_of_id[id], nsmooth, nsearch, ds);
}

int ref_smooth_one(void* h, int which, int id, const double* x, int nsmooth, const double* rho,
                   const double* smvel, const double* weight, double mean, double* out) {
    RefTree* r = (RefTree*)h;
    int ds = set_rho(r, rho);
    Double_t xx[3] = {0, 0, 0};
    if (x) for (int k = 0; k < 3; k++) xx[k] = x[k];
    int t = x ? -1 : r->tree_of_id[id];
    Double_t* w = const_cast<Double_t*>(weight);
    if (which == 0) {
        Coordinate c = x ? r->tree->CalcSmoothVelPosition(xx, nsmooth, ds)
                         : r->tree->CalcSmoothVelParticle(t, nsmooth, ds);
        for (int k = 0; k < 3; k++) out[k] = c[k];
    } else if (which == 1) {
        Coordinate sv(smvel[0], smvel[1], smvel[2]);
        Matrix m = x ? r->tree->CalcSmoothVelDispPosition(xx, sv, nsmooth, ds)
                     : r->tree->CalcSmoothVelDispParticle(t, sv, nsmooth, ds);
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) out[3 * k + l] = m(k, l);
    } else if (which == 4) {
        out[0] = x ? r->tree->CalcSmoothLocalMeanPosition(xx, w, nsmooth, ds)
                   : r->tree->CalcSmoothLocalMeanParticle(t, w, nsmooth, ds);
    } else {
        out[0] = x ? r->tree->CalcSmoothLocalDispPosition(xx, w, mean, nsmooth, ds)
                   : r->tree->CalcSmoothLocalDispParticle(t, w, mean, nsmooth, ds);
    }
    return 0;
}

}  // extern "C"
