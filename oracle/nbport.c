/*
 * Test infrastructure only: a CPU restatement of the reference NBodylib KDTree hot path.
 * It serves as the checker in tests/ (on machines where the reference itself cannot be
 * built) and as the CPU baseline in bench.py. The product library never links it.
 *
 * Each function follows the reference step by step and cites the file:line it restates.
 * The arithmetic is written in the same association order as the reference, and the
 * Makefile compiles with -ffp-contract=off, so distances, box offsets and kernel weights
 * round exactly as the reference's do. The quickselect median partition is restated
 * swap for swap, so the particle permutation (tree order) equals the reference's, which
 * tests/test_oracle.py checks against the compiled reference.
 *
 * Paths are relative to the reference checkout (pelahi/NBodylib).
 */
#include "nbport.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXVALUE 1e32 /* src/Math/Precision.h MAXVALUE */
enum { TPHYS = 0, TPROJ = 1, TVEL = 2, TPHS = 3 };
enum { KSPH = 0, KGAUSS = 1, KEPAN = 2, KTH = 3 };

typedef struct {
    double pos[3], vel[3];
    double mass, rho;
    int id, pad;
} PPart;

typedef struct {
    int start, end;   /* [start, end) in tree order */
    int left, right;  /* children; -1 for a leaf */
    int cut_dim;
    double cut_val;
    double bnd[6][2];
    double maxextent2; /* src/KDTree/KDNode.h:365-372 */
} PNode;

struct PTree {
    int n, b, treetype, nd, kerntype, kernres;
    int aniso; /* the reference's `anisotropic` flag: -1 plain phase metric, 0 local metric */
    PPart* p;
    PNode* nodes;
    int numnodes, numleaves;
    int periodic;
    double period[3];
    double* kernel;
    double kernnorm;
    int* tree_of_id;
    double build_seconds;
};

/* ---------------------------------------------------------------- priority queue */
/* 1-based binary max-heap of (index, priority): src/KDTree/PriorityQueue.h:14-85. */
typedef struct {
    int n, max_size;
    int* q;
    double* pr;
} PQ;

static void pq_init(PQ* h, int max) {
    h->n = 0;
    h->max_size = max;
    h->q = (int*)malloc(sizeof(int) * (max + 1));
    h->pr = (double*)malloc(sizeof(double) * (max + 1));
}
static void pq_free(PQ* h) {
    free(h->q);
    free(h->pr);
}
/* PriorityQueue::Push (PriorityQueue.h:47-65): sift up, stop when parent >= dist. */
static void pq_push(PQ* h, int p, double dist) {
    if (++h->n > h->max_size) abort();
    int r = h->n;
    while (r > 1) {
        int par = r >> 1;
        if (h->pr[par] >= dist) break;
        h->pr[r] = h->pr[par];
        h->q[r] = h->q[par];
        r = par;
    }
    h->pr[r] = dist;
    h->q[r] = p;
}
/* PriorityQueue::Pop (PriorityQueue.h:66-82). */
static void pq_pop(PQ* h) {
    double kn = h->pr[h->n--];
    int p = 1, r = 2;
    while (r <= h->n) {
        if (r < h->n && h->pr[r] < h->pr[r + 1]) r++;
        if (kn >= h->pr[r]) break;
        h->pr[p] = h->pr[r];
        h->q[p] = h->q[r];
        p = r;
        r = p << 1;
    }
    h->pr[p] = h->pr[h->n + 1];
    h->q[p] = h->q[h->n + 1];
}
static inline double pq_top(const PQ* h) { return h->pr[1]; }
static inline int pq_topq(const PQ* h) { return h->q[1]; }

/* ---------------------------------------------------------------- coordinates */
static inline double tcoord(const PTree* t, const PPart* a, int j) {
    if (t->treetype == TVEL) return a->vel[j];
    if (t->treetype == TPHS) return j < 3 ? a->pos[j] : a->vel[j - 3];
    return a->pos[j];
}
/* DistanceSqd with a dim loop (DistFunc.h:14-19): ((0 + dx^2) + dy^2) + dz^2 ... */
static inline double dist2_n(const double* a, const double* b, int nd) {
    double total = 0;
    for (int i = 0; i < nd; i++) total += (a[i] - b[i]) * (a[i] - b[i]);
    return total;
}
static inline void tvec(const PTree* t, const PPart* a, double* x) {
    for (int j = 0; j < t->nd; j++) x[j] = tcoord(t, a, j);
}

/* ---------------------------------------------------------------- kernel table */
static double w_sph(double r, double h) { /* SmoothingKernels.h:32-38 */
    double rh = r / h;
    if (rh <= 1.0) return (1.0 - 0.75 * (2.0 - rh) * (rh * rh));
    else if (rh > 1.0 && rh <= 2.0) return 0.25 * (2.0 - rh) * (2.0 - rh) * (2.0 - rh);
    else return 0;
}
static double w_th(double r, double h) { /* SmoothingKernels.h:40-43 */
    double rh = r / h * 0.5;
    return (rh <= 1.0);
}
static double w_gauss(double r, double h) { /* SmoothingKernels.h:45-49 */
    double rh = r / h * 2.0;
    return exp(-0.5 * pow(rh, (double)2.0));
}
static double w_epan(double r, double h) { /* SmoothingKernels.h:52-56 */
    double rh = r / h * 0.5;
    if (rh <= 1.0) return (1.0 - rh * rh);
    else return 0.;
}

/* KDTree::KernelConstruction (KDTree.cxx:1144-1183); Gamma(ND/2+1) via tgamma as the
   GSL stand-in does. */
static void kernel_construction(PTree* t) {
    if (t->kernres < 100) t->kernres = 100;
    int nd = t->nd;
    t->kernel = (double*)malloc(sizeof(double) * t->kernres);
    double kn = 1.0 / nd * pow(M_1_PI, nd / 2.) * tgamma(nd / 2. + 1.);
    double (*f)(double, double) = w_sph;
    if (t->kerntype == KSPH) {
        f = w_sph;
        kn *= nd * (nd + 1.) * (nd + 2.) * (nd + 3.) / (6 * (pow(2., nd + 1) - 1.));
    } else if (t->kerntype == KGAUSS) {
        f = w_gauss;
        kn *= pow(0.5 * M_1_PI, nd / 2.);
    } else if (t->kerntype == KEPAN) {
        f = w_epan;
        kn *= nd * (nd + 2.) * pow(0.5, nd + 1.);
    } else if (t->kerntype == KTH) {
        f = w_th;
    } else {
        f = w_sph;
        kn *= nd * (nd + 1.) * (nd + 2.) * (nd + 3.) / (6 * (pow(2., nd + 1) - 1.));
    }
    t->kernnorm = kn;
    double delta = 2.0 / (double)(t->kernres - 1);
    for (int i = 0; i < t->kernres; i++) t->kernel[i] = kn * f(i * delta, 1.0);
}

/* KDTree::Wsm (KDCalcSmoothQuantities.cxx:12-15). */
static inline double wsm(double r, int i, int size, double delta, const double* x) {
    if (i < size - 1) return (x[i] + (x[i + 1] - x[i]) * (r - delta * i) / delta);
    else return x[i];
}

/* ---------------------------------------------------------------- tree build */
/* Number of nodes in a subtree of `size` particles: the reference splits a node of
   size s > b into ceil(s/2) and floor(s/2) (KDTree.cxx:993,1012,1025,1030). */
static int subtree_nodes(int size, int b) {
    if (size <= b) return 1;
    int left = (size - 1) / 2 + 1;
    return 1 + subtree_nodes(left, b) + subtree_nodes(size - left, b);
}

/* KDTree::MedianPos/Vel/Phs, balanced branch (KDTree.cxx:328-362), restated swap for
   swap on the port's particle records. */
static double median_select(PTree* t, int d, int k, int start, int end) {
    PPart* b = t->p;
    int left = start, right = end - 1;
    while (left < right) {
        double x = tcoord(t, &b[k], d);
        PPart tmp = b[right];
        b[right] = b[k];
        b[k] = tmp;
        int pval = k;
        int i = left - 1, j = right;
        while (1) {
            while (i < j)
                if (tcoord(t, &b[++i], d) >= x) break;
            while (i < j)
                if (tcoord(t, &b[--j], d) <= x) break;
            tmp = b[i];
            b[i] = b[j];
            b[j] = tmp;
            pval = j;
            if (j <= i) break;
        }
        PPart w = b[pval];
        b[j] = b[i];
        b[i] = b[right];
        b[right] = w;
        if (i >= k) right = i - 1;
        if (i <= k) left = i + 1;
    }
    return tcoord(t, &b[k], d);
}

/* KDTree::BuildNodes (KDTree.cxx:970-1055) for the non-adaptive tree: leaf when
   size <= b; split dimension = most spread (DetermineSplitDim, :459-504, strict >);
   split index start + (size-1)/2, left = [start, split+1). Node ids are preorder, as
   BuildNodeIDs assigns them (:1185-1204). */
static void build_nodes(PTree* t, int id, int start, int end) {
    PNode* nd = &t->nodes[id];
    int size = end - start;
    nd->start = start;
    nd->end = end;
    double bnd[6][2];
    for (int j = 0; j < t->nd; j++) { /* SpreadestPos / BoundaryandMeanPos min/max */
        double mn = tcoord(t, &t->p[start], j), mx = mn;
        for (int i = start + 1; i < end; i++) {
            double v = tcoord(t, &t->p[i], j);
            if (v < mn) mn = v;
            if (v > mx) mx = v;
        }
        bnd[j][0] = mn;
        bnd[j][1] = mx;
    }
    memcpy(nd->bnd, bnd, sizeof(bnd));
    double me = 0; /* KDNode.h:368-372 */
    for (int j = 0; j < t->nd; j++) {
        double e = bnd[j][1] - bnd[j][0];
        if (e > me) me = e;
    }
    nd->maxextent2 = me * me;
    if (size <= t->b) {
        nd->left = nd->right = -1;
        nd->cut_dim = -1;
        nd->cut_val = 0;
        return;
    }
    int splitdim = 0;
    double cur = bnd[0][1] - bnd[0][0];
    for (int j = 1; j < t->nd; j++) {
        double s = bnd[j][1] - bnd[j][0];
        if (s > cur) {
            splitdim = j;
            cur = s;
        }
    }
    int splitindex = start + (size - 1) / 2;
    double splitvalue = median_select(t, splitdim, splitindex, start, end);
    nd->cut_dim = splitdim;
    nd->cut_val = splitvalue;
    int lsize = splitindex + 1 - start;
    int lid = id + 1;
    int rid = id + 1 + subtree_nodes(lsize, t->b);
    nd->left = lid;
    nd->right = rid;
    if (size > 65536) {
#pragma omp task
        build_nodes(t, lid, start, splitindex + 1);
#pragma omp task
        build_nodes(t, rid, splitindex + 1, end);
#pragma omp taskwait
    } else {
        build_nodes(t, lid, start, splitindex + 1);
        build_nodes(t, rid, splitindex + 1, end);
    }
}

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

PTree* pt_create(const double* pos, const double* vel, const double* mass, int n, int b,
                 int treetype, int kerntype, int kernres, const double* period, int nthreads) {
    PTree* t = (PTree*)calloc(1, sizeof(PTree));
    t->n = n;
    t->b = b;
    t->treetype = treetype;
    t->kerntype = kerntype;
    t->kernres = kernres;
    t->nd = (treetype == TPHS) ? 6 : (treetype == TPROJ ? 2 : 3);
    if (period) {
        t->periodic = 1;
        for (int k = 0; k < 3; k++) t->period[k] = period[k];
    }
    kernel_construction(t);
    t->p = (PPart*)malloc(sizeof(PPart) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        PPart* q = &t->p[i];
        for (int j = 0; j < 3; j++) {
            q->pos[j] = pos[3 * i + j];
            q->vel[j] = vel ? vel[3 * i + j] : 0.0;
        }
        q->mass = mass ? mass[i] : 1.0;
        q->rho = 0;
        q->id = i; /* KDTree.cxx:1291 */
        q->pad = 0;
    }
    int nn = subtree_nodes(n, b);
    t->nodes = (PNode*)calloc((size_t)nn, sizeof(PNode));
    t->numnodes = nn;
    double t0 = now_seconds();
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#pragma omp single
#endif
    build_nodes(t, 0, 0, n);
    t->build_seconds = now_seconds() - t0;
    t->numleaves = 0;
    for (int i = 0; i < nn; i++)
        if (t->nodes[i].left < 0) t->numleaves++;
    t->tree_of_id = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) t->tree_of_id[t->p[i].id] = i;
    return t;
}

void pt_destroy(PTree* t) {
    if (!t) return;
    free(t->p);
    free(t->nodes);
    free(t->kernel);
    free(t->tree_of_id);
    free(t);
}
void pt_set_aniso(PTree* t, int aniso) { t->aniso = aniso; }
int pt_num_nodes(const PTree* t) { return t->numnodes; }
int pt_num_leaves(const PTree* t) { return t->numleaves; }
double pt_kernnorm(const PTree* t) { return t->kernnorm; }
double pt_build_seconds(const PTree* t) { return t->build_seconds; }
void pt_kernel_table(const PTree* t, double* table) {
    memcpy(table, t->kernel, sizeof(double) * t->kernres);
}
void pt_ids(const PTree* t, int* ids) {
    for (int i = 0; i < t->n; i++) ids[i] = t->p[i].id;
}
void pt_leaf_start(const PTree* t, int* ls) {
    for (int i = 0; i < t->numnodes; i++)
        if (t->nodes[i].left < 0)
            for (int j = t->nodes[i].start; j < t->nodes[i].end; j++) ls[j] = t->nodes[i].start;
}

/* ---------------------------------------------------------------- kNN */
/* SplitNode::FindNearestPos(target) (KDSplitNode.cxx:15-41) and
   LeafNode::FindNearestPos(target) (KDLeafNode.cxx:15-28): excludes the target and any
   particle at distance 0. Generalised over the tree's coordinate space (Vel, Phase). */
static void knn_target(const PTree* t, int node, double rd, PQ* pq, double* off, int target,
                       const double* xt) {
    const PNode* nd = &t->nodes[node];
    if (nd->left < 0) {
        double xi[6];
        for (int i = nd->start; i < nd->end; i++) {
            if (i != target) {
                tvec(t, &t->p[i], xi);
                double d2 = dist2_n(xt, xi, t->nd);
                if (d2 < pq_top(pq) && d2 > 0) {
                    pq_pop(pq);
                    pq_push(pq, i, d2);
                }
            }
        }
        return;
    }
    int cd = nd->cut_dim;
    double old_off = off[cd];
    double new_off = xt[cd] - nd->cut_val;
    if (new_off < 0) {
        knn_target(t, nd->left, rd, pq, off, target, xt);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < pq_top(pq)) {
            off[cd] = new_off;
            knn_target(t, nd->right, rd, pq, off, target, xt);
            off[cd] = old_off;
        }
    } else {
        knn_target(t, nd->right, rd, pq, off, target, xt);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < pq_top(pq)) {
            off[cd] = new_off;
            knn_target(t, nd->left, rd, pq, off, target, xt);
            off[cd] = old_off;
        }
    }
}

/* FindNearestPos(x) (KDSplitNode.cxx:206-231, KDLeafNode.cxx:119-130): coordinate
   search, nothing excluded. */
static void knn_coord(const PTree* t, int node, double rd, PQ* pq, double* off, const double* x) {
    const PNode* nd = &t->nodes[node];
    if (nd->left < 0) {
        double xi[6];
        for (int i = nd->start; i < nd->end; i++) {
            tvec(t, &t->p[i], xi);
            double d2 = dist2_n(x, xi, t->nd);
            if (d2 < pq_top(pq)) {
                pq_pop(pq);
                pq_push(pq, i, d2);
            }
        }
        return;
    }
    int cd = nd->cut_dim;
    double old_off = off[cd];
    double new_off = x[cd] - nd->cut_val;
    if (new_off < 0) {
        knn_coord(t, nd->left, rd, pq, off, x);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < pq_top(pq)) {
            off[cd] = new_off;
            knn_coord(t, nd->right, rd, pq, off, x);
            off[cd] = old_off;
        }
    } else {
        knn_coord(t, nd->right, rd, pq, off, x);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < pq_top(pq)) {
            off[cd] = new_off;
            knn_coord(t, nd->left, rd, pq, off, x);
            off[cd] = old_off;
        }
    }
}

/* PeriodicReflection1D/2D/ND (DistFunc.h:326-355). Returns sval; writes the image. */
static double reflect(const double* x0, double* xp, const double* p, int mask) {
    double s = 0;
    int cnt = 0, only = -1;
    for (int k = 0; k < 3; k++) xp[k] = x0[k];
    for (int k = 0; k < 3; k++) {
        if (!(mask >> k & 1)) continue;
        cnt++;
        only = k;
    }
    if (cnt == 1) {
        int k = only;
        if (x0[k] < p[k] / 2.0) {
            xp[k] = x0[k] + p[k];
            s = x0[k];
        } else {
            xp[k] = x0[k] - p[k];
            s = -xp[k];
        }
        return s;
    }
    for (int k = 0; k < 3; k++) {
        if (!(mask >> k & 1)) continue;
        if (x0[k] < p[k] / 2.0) {
            xp[k] = x0[k] + p[k];
            s += x0[k] * x0[k];
        } else {
            xp[k] = x0[k] - p[k];
            s += xp[k] * xp[k];
        }
    }
    return sqrt(s);
}
/* The image order the reference searches: x, y, z, xy, xz, yz, xyz
   (KDSplitNode.cxx:1126-1147). */
static const int kImageMask[7] = {1, 2, 4, 3, 5, 6, 7};

/* SplitNode::FindNearestPosPeriodic(x) (KDSplitNode.cxx:1119-1147), including its gate
   mismatch: 1-D images are gated by sqrt(top) > sval, 2-D/3-D images by top > sval. */
static void knn_periodic(const PTree* t, PQ* pq, const double* x) {
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xp[3];
    knn_coord(t, 0, 0.0, pq, off, x);
    for (int m = 0; m < 7; m++) {
        for (int j = 0; j < 6; j++) off[j] = 0.0;
        double sval = reflect(x, xp, t->period, kImageMask[m]);
        int gate = (m < 3) ? (sqrt(pq_top(pq)) > sval) : (pq_top(pq) > sval);
        if (gate) knn_coord(t, 0, 0.0, pq, off, xp);
    }
}

/* MetricDistSqd (DistFunc.h:58-65): over the six phase coordinates, total += metric[i]*d*d
   from 0 in dimension order. */
static inline double metric_dist2(const double* a, const double* b, const double* metric) {
    double total = 0;
    for (int i = 0; i < 6; i++) total += metric[i] * (a[i] - b[i]) * (a[i] - b[i]);
    return total;
}

/* SplitNode::FindNearestMetric (KDSplitNode.cxx:96-121 target form, 303-331 coordinate
   form) and LeafNode::FindNearestMetric (KDLeafNode.cxx:58-71, 168-179). The leaves test
   the metric distance while the pruning test compares the unscaled incremental offset rd
   with the heap top, so the search is not exact and its result depends on the traversal
   order, which this restatement keeps. target < 0: the coordinate form. Both forms skip
   distance 0; the target form also skips the target. */
static void knn_metric(const PTree* t, int node, double rd, PQ* pq, double* off, int target,
                       const double* x, const double* metric) {
    const PNode* nd = &t->nodes[node];
    if (nd->left < 0) {
        double xi[6];
        for (int i = nd->start; i < nd->end; i++) {
            if (i == target) continue;
            tvec(t, &t->p[i], xi);
            double d2 = metric_dist2(x, xi, metric);
            if (d2 < pq_top(pq) && d2 > 0) {
                pq_pop(pq);
                pq_push(pq, i, d2);
            }
        }
        return;
    }
    int cd = nd->cut_dim;
    double old_off = off[cd];
    double new_off = x[cd] - nd->cut_val;
    if (new_off < 0) {
        knn_metric(t, nd->left, rd, pq, off, target, x, metric);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < pq_top(pq)) {
            off[cd] = new_off;
            knn_metric(t, nd->right, rd, pq, off, target, x, metric);
            off[cd] = old_off;
        }
    } else {
        knn_metric(t, nd->right, rd, pq, off, target, x, metric);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < pq_top(pq)) {
            off[cd] = new_off;
            knn_metric(t, nd->left, rd, pq, off, target, x, metric);
            off[cd] = old_off;
        }
    }
}

static void phase_periodic(const PTree* t, PQ* pq, const double* x, const double* metric);

/* KDTree::CalculateMetricSpacing: the 8 nearest in plain phase space around x (coordinate
   search: a particle at x itself is included), popped into ID[7..0]; the six direct
   offsets to ID[1] (or to the next one if their product is 0) give metric[j] =
   1/sr0[j]^2. The reference defines this inline function twice: the copy in
   KDCalcSmoothQuantities.cxx:17-56, which the density functions use, always searches
   without images; the copy in KDFindNearest.cxx:34-105, which FindNearest uses, searches
   the periodic images of a periodic tree (FindNearestPhasePeriodic). `periodic` selects
   the latter. Returns 6 when fewer than 8 particles exist (the reference exits). */
static int metric_spacing(const PTree* t, const double* x, double* metric, int periodic) {
    PQ pq;
    pq_init(&pq, 8);
    for (int i = 0; i < 8; i++) pq_push(&pq, -1, MAXVALUE);
    double off[6] = {0, 0, 0, 0, 0, 0};
    if (periodic) phase_periodic(t, &pq, x, NULL);
    else knn_coord(t, 0, 0.0, &pq, off, x);
    int id[8];
    for (int i = 7; i >= 0; i--) {
        id[i] = pq_topq(&pq);
        if (id[i] == -1) {
            pq_free(&pq);
            return 6;
        }
        pq_pop(&pq);
    }
    pq_free(&pq);
    double kvol = 0.0, sr0[6] = {0, 0, 0, 0, 0, 0};
    int ivol = 1;
    while (kvol == 0.0 && ivol < 8) {
        kvol = 1.0;
        for (int j = 0; j < 6; j++) {
            const PPart* a = &t->p[id[ivol]];
            sr0[j] = fabs((j < 3 ? a->pos[j] : a->vel[j - 3]) - x[j]);
            kvol *= sr0[j];
        }
        ivol++;
    }
    for (int j = 0; j < 6; j++) metric[j] = 1.0 / (sr0[j] * sr0[j]);
    return 0;
}

/* SplitNode::FindNearestPhasePeriodic / FindNearestMetricPeriodic (KDSplitNode.cxx:
   1153-1186, 1193-1218): the coordinate search around x (position and velocity), then the
   seven position images x, y, z, xy, xz, yz, xyz with no gate, the offsets reset before
   each. metric == NULL: plain phase distance. A root that is a leaf searches x alone
   (KDLeafNode.cxx:666-679, 708-711, 725-728). */
static void phase_periodic(const PTree* t, PQ* pq, const double* x, const double* metric) {
    double off[6] = {0, 0, 0, 0, 0, 0};
    if (metric) knn_metric(t, 0, 0.0, pq, off, -1, x, metric);
    else knn_coord(t, 0, 0.0, pq, off, x);
    if (t->nodes[0].left < 0) return;
    for (int m = 0; m < 7; m++) {
        double xp[6];
        for (int j = 0; j < 6; j++) off[j] = 0.0;
        reflect(x, xp, t->period, kImageMask[m]);
        for (int j = 3; j < 6; j++) xp[j] = x[j];
        if (metric) knn_metric(t, 0, 0.0, pq, off, -1, xp, metric);
        else knn_coord(t, 0, 0.0, pq, off, xp);
    }
}

/* LoadNN (KDFindNearest.cxx:11-24): pop the ns largest into nn[ns-1..0]. */
static void load_nn(const PTree* t, int ns, PQ* pq, int* nn, double* d) {
    for (int i = ns - 1; i >= 0; i--) {
        int q = pq_topq(pq);
        nn[i] = q >= 0 ? t->p[q].id : -1;
        d[i] = pq_top(pq);
        pq_pop(pq);
    }
}

/* The search KDTree::FindNearest(tt) runs for the tree's type (KDFindNearest.cxx:
   255-310): physical trees the target search or the gated periodic one; velocity trees
   the target search even when periodic; phase-space trees the plain phase search
   (anisotropic -1) or the local-metric search (0), each with its ungated periodic form.
   xt: the target's tree coordinates. Returns 6 when the metric spacing fails. */
static int search_target(const PTree* t, PQ* pq, int tt, const double* xt) {
    double off[6] = {0, 0, 0, 0, 0, 0};
    int per = t->periodic;
    if (t->treetype == TPHS) {
        if (t->aniso == -1) {
            if (!per) knn_target(t, 0, 0.0, pq, off, tt, xt);
            else phase_periodic(t, pq, xt, NULL);
        } else {
            double m[6];
            if (metric_spacing(t, xt, m, per)) return 6;
            if (!per) knn_metric(t, 0, 0.0, pq, off, tt, xt, m);
            else phase_periodic(t, pq, xt, m);
        }
        return 0;
    }
    int root_leaf = t->nodes[0].left < 0;
    if (!per || root_leaf || t->treetype == TVEL) knn_target(t, 0, 0.0, pq, off, tt, xt);
    else knn_periodic(t, pq, xt);
    return 0;
}

/* KDTree::FindNearest(tt) / FindNearestPos(tt) (KDFindNearest.cxx:247-334). method 0:
   FindNearest, 1: FindNearestPos (physical trees only). A periodic tree searches for k+1
   (any tree type, :250) and then loads k: FindNearest drops the nearest entry,
   FindNearestPos pops the farthest first (:331). */
static int find_nearest_one(const PTree* t, int method, int tt, int k, PQ* pq, int* nn, double* d) {
    int ns = k;
    int per = t->periodic;
    if (per) ns += 1;
    pq->n = 0;
    for (int i = 0; i < ns; i++) pq_push(pq, -1, MAXVALUE);
    double xt[6] = {0, 0, 0, 0, 0, 0};
    tvec(t, &t->p[tt], xt);
    int st = search_target(t, pq, tt, xt);
    if (per) {
        if (method == 1) pq_pop(pq);
        ns -= 1;
    }
    load_nn(t, ns, pq, nn, d);
    return st;
}

int pt_knn(PTree* t, int method, int k, int nthreads, int* nn_ids, double* d2) {
    int n = t->n;
    if (method == 1 && t->treetype != TPHYS) return 7;
    int status = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        PQ pq;
        pq_init(&pq, k + 1);
#ifdef _OPENMP
#pragma omp for schedule(guided)
#endif
        for (int id = 0; id < n; id++) {
            int tt = t->tree_of_id[id];
            if (find_nearest_one(t, method, tt, k, &pq, nn_ids + (size_t)id * k,
                                 d2 + (size_t)id * k))
                status = 6;
        }
        pq_free(&pq);
    }
    return status;
}

/* KDTree::FindNearestPos(Double_t *x) (KDFindNearest.cxx:509-520). */
int pt_knn_pos(PTree* t, const double* x, int nq, int k, int nthreads, int* nn_ids, double* d2) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        PQ pq;
        pq_init(&pq, k);
#ifdef _OPENMP
#pragma omp for schedule(guided)
#endif
        for (int q = 0; q < nq; q++) {
            pq.n = 0;
            for (int i = 0; i < k; i++) pq_push(&pq, -1, MAXVALUE);
            double off[6] = {0, 0, 0, 0, 0, 0};
            const double* xq = x + 3 * (size_t)q;
            if (!t->periodic || t->nodes[0].left < 0) knn_coord(t, 0, 0.0, &pq, off, xq);
            else knn_periodic(t, &pq, xq);
            load_nn(t, k, &pq, nn_ids + (size_t)q * k, d2 + (size_t)q * k);
        }
        pq_free(&pq);
    }
    return 0;
}

/* KDTree::FindNearest(Double_t *x) (KDFindNearest.cxx:460-507): x holds the tree's
   coordinates (3 positions, 3 velocities, or 6 phase coordinates per row); nothing is
   excluded except, in the local-metric search, distance 0. Periodic velocity trees are
   not restated (returns 7). */
int pt_knn_coord(PTree* t, const double* x, int nq, int k, int nthreads, int* nn_ids, double* d2) {
    if (t->periodic && t->treetype == TVEL) return 7;
    int nd = t->nd, status = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        PQ pq;
        pq_init(&pq, k);
#ifdef _OPENMP
#pragma omp for schedule(guided)
#endif
        for (int q = 0; q < nq; q++) {
            pq.n = 0;
            for (int i = 0; i < k; i++) pq_push(&pq, -1, MAXVALUE);
            double off[6] = {0, 0, 0, 0, 0, 0};
            const double* xq = x + (size_t)nd * q;
            if (t->treetype == TPHS) {
                double m[6];
                if (t->aniso == -1) {
                    if (!t->periodic) knn_coord(t, 0, 0.0, &pq, off, xq);
                    else phase_periodic(t, &pq, xq, NULL);
                } else if (metric_spacing(t, xq, m, t->periodic)) {
                    status = 6;
                } else if (!t->periodic) {
                    knn_metric(t, 0, 0.0, &pq, off, -1, xq, m);
                } else {
                    phase_periodic(t, &pq, xq, m);
                }
            } else if (!t->periodic || t->nodes[0].left < 0) {
                knn_coord(t, 0, 0.0, &pq, off, xq);
            } else {
                knn_periodic(t, &pq, xq);
            }
            load_nn(t, k, &pq, nn_ids + (size_t)q * k, d2 + (size_t)q * k);
        }
        pq_free(&pq);
    }
    return status;
}

/* The neighbour search of CalcDensity / CalcDensityParticle for the tree's type
   (KDCalcSmoothQuantities.cxx:227-263, 782-816): always non-periodic. For a phase-space
   tree with the local metric, *scale receives the product of sqrt(metric[j]) that
   multiplies the normalisation (:265-270); otherwise 1. Returns 7 for a phase-space tree
   without the local metric (the reference multiplies uninitialised metric arrays there),
   6 when the metric spacing fails. */
static int density_search(const PTree* t, PQ* pq, int i, double* scale) {
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xt[6] = {0, 0, 0, 0, 0, 0};
    tvec(t, &t->p[i], xt);
    *scale = 1.0;
    if (t->treetype != TPHS) {
        knn_target(t, 0, 0.0, pq, off, i, xt);
        return 0;
    }
    if (t->aniso != 0) return 7;
    double m[6];
    if (metric_spacing(t, xt, m, 0)) return 6;
    knn_metric(t, 0, 0.0, pq, off, i, xt, m);
    double temp = 1.0;
    for (int j = 0; j < 6; j++) m[j] = sqrt(m[j]);
    for (int j = 0; j < 6; j++) temp *= m[j];
    *scale = temp;
    return 0;
}

/* ---------------------------------------------------------------- SPH density */
/* KDTree::CalcDensity (KDCalcSmoothQuantities.cxx:203-305): non-periodic target search
   (density_search) for every particle in tree order; h = 0.5 sqrt(top), norm = h^-ND
   (times the metric factor of a phase-space tree); symmetric scatter. Returns 6 when a
   neighbour slot stays empty (the reference calls exit(1), :273-276), 7 for a phase-space
   tree without the local metric. */
int pt_density(PTree* t, int k, double* rho, int* nn_ids) {
    int n = t->n;
    for (int i = 0; i < n; i++) t->p[i].rho = 0;
    PQ pq;
    pq_init(&pq, k);
    int nd = t->nd;
    double delta = 2.0 / (double)(t->kernres - 1);
    int status = 0;
    for (int i = 0; i < n && !status; i++) {
        pq.n = 0;
        for (int j = 0; j < k; j++) pq_push(&pq, -1, MAXVALUE);
        double scale;
        status = density_search(t, &pq, i, &scale);
        if (status) break;
        double hi = 0.5 * sqrt(pq_top(&pq));
        double norm = 1.0 / pow(hi, (double)(nd * 1.));
        if (t->treetype == TPHS) norm *= scale;
        for (int j = 0; j < k; j++) {
            if (pq_topq(&pq) == -1) {
                status = 6;
                break;
            }
            double rij = sqrt(pq_top(&pq));
            double wij = 0.5 * wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres,
                                   delta, t->kernel) *
                         norm;
            int id = pq_topq(&pq);
            if (nn_ids) nn_ids[(size_t)t->p[i].id * k + j] = t->p[id].id;
            t->p[i].rho = t->p[i].rho + wij * t->p[id].mass;
            t->p[id].rho = t->p[id].rho + wij * t->p[i].mass;
            pq_pop(&pq);
        }
    }
    pq_free(&pq);
    for (int i = 0; i < n; i++) rho[t->p[i].id] = t->p[i].rho;
    return status;
}

/* KDTree::CalcVelDensity (KDCalcSmoothQuantities.cxx:309-389), physical tree. */
static double veldensity_one(PTree* t, int i, int nsmooth, int nsearch, PQ* pq, PQ* pq2,
                             int* nnids, double* vdist, int* status) {
    int nd = t->nd;
    double delta = 2.0 / (double)(t->kernres - 1);
    pq->n = 0;
    for (int j = 0; j < nsearch; j++) pq_push(pq, -1, MAXVALUE);
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xt[6] = {0, 0, 0, 0, 0, 0};
    tvec(t, &t->p[i], xt);
    knn_target(t, 0, 0.0, pq, off, i, xt);
    for (int j = 0; j < nsearch; j++) {
        if (pq_topq(pq) == -1) {
            *status = 6;
            return 0;
        }
        nnids[j] = pq_topq(pq);
        /* VelDistSqd(v1, v2, ND) (DistFunc.h:21-26) */
        vdist[j] = sqrt(dist2_n(t->p[i].vel, t->p[nnids[j]].vel, nd < 3 ? nd : 3));
        pq_pop(pq);
    }
    pq2->n = 0;
    for (int j = 0; j < nsmooth; j++) pq_push(pq2, -1, MAXVALUE);
    for (int j = 0; j < nsearch; j++)
        if (vdist[j] < pq_top(pq2)) {
            pq_pop(pq2);
            pq_push(pq2, nnids[j], vdist[j]);
        }
    double hi = 0.5 * pq_top(pq2);
    double norm = 1.0 / pow(hi, (double)(nd * 1.));
    double den = 0;
    for (int j = 0; j < nsmooth; j++) {
        double rij = pq_top(pq2);
        double wij =
            wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres, delta, t->kernel) *
            norm;
        den = den + wij;
        pq_pop(pq2);
    }
    return den;
}

int pt_veldensity(PTree* t, int nsmooth, int nsearch, double* out) {
    if (nsmooth > nsearch) nsmooth = nsearch;
    int n = t->n;
    int status = 0;
    PQ pq, pq2;
    pq_init(&pq, nsearch);
    pq_init(&pq2, nsmooth);
    int* nnids = (int*)malloc(sizeof(int) * nsearch);
    double* vdist = (double*)malloc(sizeof(double) * nsearch);
    for (int i = 0; i < n && !status; i++)
        out[t->p[i].id] = veldensity_one(t, i, nsmooth, nsearch, &pq, &pq2, nnids, vdist, &status);
    free(nnids);
    free(vdist);
    pq_free(&pq);
    pq_free(&pq2);
    return status;
}

/* pt_density with the per-particle searches spread over OpenMP threads, for checking
   large particle sets in reasonable time (the reference's CalcDensity is a serial loop).
   Each particle's search, smoothing length and weights are exactly those of pt_density;
   the symmetric scatter goes to one accumulator per thread (static schedule), summed at
   the end, so a density differs from pt_density's only by the order in which its
   non-negative terms are added (a few ulps). Physical and velocity trees only. */
int pt_density_parallel(PTree* t, int k, int nthreads, double* rho) {
    int n = t->n;
    if (t->treetype == TPHS) return 7;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    int nt = omp_get_max_threads();
    double* acc = (double*)calloc((size_t)nt * n, sizeof(double));
    if (!acc) return 8;
    int nd = t->nd;
    double delta = 2.0 / (double)(t->kernres - 1);
    int status = 0;
#pragma omp parallel
    {
        PQ pq;
        pq_init(&pq, k);
        double* my = acc + (size_t)omp_get_thread_num() * n;
#pragma omp for schedule(static, 256)
        for (int i = 0; i < n; i++) {
            pq.n = 0;
            for (int j = 0; j < k; j++) pq_push(&pq, -1, MAXVALUE);
            double scale;
            density_search(t, &pq, i, &scale);
            double hi = 0.5 * sqrt(pq_top(&pq));
            double norm = 1.0 / pow(hi, (double)(nd * 1.));
            for (int j = 0; j < k; j++) {
                if (pq_topq(&pq) == -1) {
#pragma omp atomic write
                    status = 6;
                    break;
                }
                double rij = sqrt(pq_top(&pq));
                double wij = 0.5 *
                             wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres,
                                 delta, t->kernel) *
                             norm;
                int id = pq_topq(&pq);
                my[i] += wij * t->p[id].mass;
                my[id] += wij * t->p[i].mass;
                pq_pop(&pq);
            }
        }
        pq_free(&pq);
#pragma omp for schedule(static)
        for (int i = 0; i < n; i++) {
            double s = 0;
            for (int th = 0; th < nt; th++) s += acc[(size_t)th * n + i];
            rho[t->p[i].id] = s;
        }
    }
    free(acc);
    return status;
}

/* pt_veldensity with the particles spread over OpenMP threads: every value is a gather
   over the particle's own neighbours, so the results are bit-identical to pt_veldensity. */
int pt_veldensity_parallel(PTree* t, int nsmooth, int nsearch, int nthreads, double* out) {
    if (nsmooth > nsearch) nsmooth = nsearch;
    int n = t->n;
    int status = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
    {
        PQ pq, pq2;
        pq_init(&pq, nsearch);
        pq_init(&pq2, nsmooth);
        int* nnids = (int*)malloc(sizeof(int) * nsearch);
        double* vdist = (double*)malloc(sizeof(double) * nsearch);
        int st = 0;
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < n; i++)
            out[t->p[i].id] = veldensity_one(t, i, nsmooth, nsearch, &pq, &pq2, nnids, vdist, &st);
        if (st) {
#pragma omp atomic write
            status = st;
        }
        free(nnids);
        free(vdist);
        pq_free(&pq);
        pq_free(&pq2);
    }
    return status;
}

/* KDTree::CalcDensityParticle (KDCalcSmoothQuantities.cxx:768-843): gather only,
   no 0.5 factor, no scatter. */
double pt_density_particle(PTree* t, int id, int k) {
    int i = t->tree_of_id[id];
    PQ pq;
    pq_init(&pq, k);
    for (int j = 0; j < k; j++) pq_push(&pq, -1, MAXVALUE);
    double scale;
    if (density_search(t, &pq, i, &scale)) {
        pq_free(&pq);
        return NAN;
    }
    double delta = 2.0 / (double)(t->kernres - 1);
    double hi = 0.5 * sqrt(pq_top(&pq));
    double norm = 1.0 / pow(hi, (double)(t->nd * 1.));
    if (t->treetype == TPHS) norm *= scale;
    double den = 0.;
    for (int j = 0; j < k; j++) {
        if (pq_topq(&pq) == -1) {
            den = NAN;
            break;
        }
        double rij = sqrt(pq_top(&pq));
        double wij =
            wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres, delta, t->kernel) *
            norm;
        den += wij * t->p[pq_topq(&pq)].mass;
        pq_pop(&pq);
    }
    pq_free(&pq);
    return den;
}

double pt_veldensity_particle(PTree* t, int id, int nsmooth, int nsearch) {
    if (nsmooth > nsearch) nsmooth = nsearch;
    PQ pq, pq2;
    pq_init(&pq, nsearch);
    pq_init(&pq2, nsmooth);
    int* nnids = (int*)malloc(sizeof(int) * nsearch);
    double* vdist = (double*)malloc(sizeof(double) * nsearch);
    int status = 0;
    double v = veldensity_one(t, t->tree_of_id[id], nsmooth, nsearch, &pq, &pq2, nnids, vdist,
                              &status);
    free(nnids);
    free(vdist);
    pq_free(&pq);
    pq_free(&pq2);
    return status ? NAN : v;
}

/* KDTree::CalcDensityPosition (KDCalcSmoothQuantities.cxx:1092-1148) for physical trees:
   the coordinate search (FindNearestPos(x): nothing excluded, never periodic), then the
   gather of CalcDensityParticle with the particle masses. NAN when fewer than k particles
   exist, and for other tree types: for velocity trees the reference multiplies the
   normalisation by metric factors it never sets (:1125-1130); phase-space trees are not
   restated. */
double pt_density_position(PTree* t, const double* x, int k) {
    if (t->treetype != TPHYS) return NAN;
    PQ pq;
    pq_init(&pq, k);
    for (int j = 0; j < k; j++) pq_push(&pq, -1, MAXVALUE);
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xq[6] = {x[0], x[1], x[2], 0, 0, 0};
    knn_coord(t, 0, 0.0, &pq, off, xq);
    double delta = 2.0 / (double)(t->kernres - 1);
    double hi = 0.5 * sqrt(pq_top(&pq));
    double norm = 1.0 / pow(hi, (double)(t->nd * 1.));
    double den = 0.;
    for (int j = 0; j < k; j++) {
        if (pq_topq(&pq) == -1) {
            den = NAN;
            break;
        }
        double rij = sqrt(pq_top(&pq));
        double wij =
            wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres, delta, t->kernel) *
            norm;
        den += wij * t->p[pq_topq(&pq)].mass;
        pq_pop(&pq);
    }
    pq_free(&pq);
    return den;
}

/* KDTree::CalcVelDensityPosition (KDCalcSmoothQuantities.cxx:1149-1207), physical tree:
   FindNearestPos(x) with nsearch, |v - v_j| for the given velocity v, the nsmooth smallest
   kept, h = 0.5 max, unit weights. NAN as above or for a non-physical tree. */
double pt_veldensity_position(PTree* t, const double* x, const double* v, int nsmooth,
                              int nsearch) {
    if (t->treetype != TPHYS) return NAN;
    if (nsmooth > nsearch) nsmooth = nsearch;
    PQ pq, pq2;
    pq_init(&pq, nsearch);
    pq_init(&pq2, nsmooth);
    for (int j = 0; j < nsearch; j++) pq_push(&pq, -1, MAXVALUE);
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xq[6] = {x[0], x[1], x[2], 0, 0, 0};
    knn_coord(t, 0, 0.0, &pq, off, xq);
    int* nnids = (int*)malloc(sizeof(int) * (size_t)nsearch);
    double* vdist = (double*)malloc(sizeof(double) * (size_t)nsearch);
    double vden = 0.;
    int bad = 0;
    for (int j = 0; j < nsearch; j++) {
        if (pq_topq(&pq) == -1) {
            bad = 1;
            break;
        }
        nnids[j] = pq_topq(&pq);
        vdist[j] = sqrt(dist2_n(v, t->p[nnids[j]].vel, 3));
        pq_pop(&pq);
    }
    if (!bad) {
        for (int j = 0; j < nsmooth; j++) pq_push(&pq2, -1, MAXVALUE);
        for (int j = 0; j < nsearch; j++)
            if (vdist[j] < pq_top(&pq2)) {
                pq_pop(&pq2);
                pq_push(&pq2, nnids[j], vdist[j]);
            }
        double delta = 2.0 / (double)(t->kernres - 1);
        double hi = 0.5 * pq_top(&pq2);
        double norm = 1.0 / pow(hi, (double)(t->nd * 1.));
        for (int j = 0; j < nsmooth; j++) {
            double rij = pq_top(&pq2);
            vden += wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres, delta,
                        t->kernel) *
                    norm;
            pq_pop(&pq2);
        }
    }
    free(nnids);
    free(vdist);
    pq_free(&pq);
    pq_free(&pq2);
    return bad ? NAN : vden;
}

/* ---------------------------------------------------------------- ball search */
/* Node::__checkboundaries (KDNode.h:280-291) as FlagNodeForSearchBallPos /
   FlagNodeForFOFSearchBall use it for non-adaptive trees (farthest2 = -1):
   1 when the farthest box corner is closer than fdist. */
static int check_boundaries(const PNode* nd, int numdim, const double* x, double fdist2) {
    double maxr2 = 0;
    for (int j = 0; j < numdim; j++) {
        double da = x[j] - nd->bnd[j][0], db = nd->bnd[j][1] - x[j];
        double da2 = da * da, db2 = db * db;
        maxr2 += da2 > db2 ? da2 : db2;
    }
    return maxr2 < fdist2;
}
/* FlagNodeForSearchBallPos / FlagNodeForFOFSearchBall (KDNode.h:294-332). */
static int flag_node(const PNode* nd, int numdim, const double* x, double fdist2) {
    if (nd->maxextent2 > fdist2) return 0;
    return check_boundaries(nd, numdim, x, fdist2);
}
/* LeafNode whole-bucket test (KDLeafNode.cxx:250-255): no maxextent2 condition. */
static int leaf_enclosed(const PNode* nd, int numdim, const double* x, double fdist2) {
    double maxr2 = 0.0;
    for (int j = 0; j < numdim; j++) {
        double a = fabs(x[j] - nd->bnd[j][0]), c = fabs(x[j] - nd->bnd[j][1]);
        double m = a > c ? a : c;
        maxr2 += m * m;
    }
    return maxr2 < fdist2;
}

typedef struct {
    int* out;
    int cnt;
    int* mark;
    double* dist2;
    int imark;
} BallOut;

static void ball_emit(const PTree* t, BallOut* o, int i, double d2) {
    if (o->mark) {
        int id = t->p[i].id;
        o->mark[id] = o->imark;
        o->dist2[id] = d2;
    } else {
        o->out[o->cnt++] = t->p[i].id;
    }
}

/* SearchBallPos / SearchBallPosTagged node recursion (KDSplitNode.cxx:455-534,
   600-690; KDLeafNode.cxx:247-410). target < 0 means the coordinate version. `tagged`
   selects the Tagged flavour, whose target version excludes the target everywhere. */
static void ball_rec(const PTree* t, int node, double rd, double fdist2, double* off,
                     const double* x, int target, int tagged, BallOut* o) {
    const PNode* nd = &t->nodes[node];
    int nd3 = t->nd;
    if (nd->left < 0) {
        if (leaf_enclosed(nd, nd3, x, fdist2)) {
            for (int i = nd->start; i < nd->end; i++) {
                if (tagged && target >= 0 && i == target) continue;
                double xi[6];
                tvec(t, &t->p[i], xi);
                ball_emit(t, o, i, o->mark ? dist2_n(x, xi, nd3) : 0.0);
            }
        } else {
            for (int i = nd->start; i < nd->end; i++) {
                if (target >= 0 && i == target) continue;
                double xi[6];
                tvec(t, &t->p[i], xi);
                double d2 = dist2_n(x, xi, nd3);
                if (d2 < fdist2) ball_emit(t, o, i, d2);
            }
        }
        return;
    }
    int fl = flag_node(nd, nd3, x, fdist2);
    if (fl == 1) {
        for (int i = nd->start; i < nd->end; i++) {
            if (tagged && target >= 0 && i == target) continue;
            double xi[6];
            tvec(t, &t->p[i], xi);
            ball_emit(t, o, i, o->mark ? dist2_n(x, xi, nd3) : 0.0);
        }
        return;
    }
    int cd = nd->cut_dim;
    double old_off = off[cd];
    double new_off = x[cd] - nd->cut_val;
    if (new_off < 0) {
        ball_rec(t, nd->left, rd, fdist2, off, x, target, tagged, o);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < fdist2) {
            off[cd] = new_off;
            ball_rec(t, nd->right, rd, fdist2, off, x, target, tagged, o);
            off[cd] = old_off;
        }
    } else {
        ball_rec(t, nd->right, rd, fdist2, off, x, target, tagged, o);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < fdist2) {
            off[cd] = new_off;
            ball_rec(t, nd->left, rd, fdist2, off, x, target, tagged, o);
            off[cd] = old_off;
        }
    }
}

/* SearchBallPos[Tagged]Periodic(x) (KDSplitNode.cxx:1348-1373, 1389-1414): direct search
   plus every image whose wall distance is below the radius (fdist2 > sval^2). */
static void ball_periodic(const PTree* t, double fdist2, const double* x, int tagged, BallOut* o) {
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xp[3];
    ball_rec(t, 0, 0.0, fdist2, off, x, -1, tagged, o);
    for (int m = 0; m < 7; m++) {
        for (int j = 0; j < 6; j++) off[j] = 0.0;
        double sval = reflect(x, xp, t->period, kImageMask[m]);
        if (fdist2 > sval * sval) ball_rec(t, 0, 0.0, fdist2, off, xp, -1, tagged, o);
    }
}

int pt_ball_tagged(PTree* t, int id, double fdist2, int* out_ids) {
    BallOut o = {out_ids, 0, NULL, NULL, 0};
    int tt = t->tree_of_id[id];
    double x[6];
    tvec(t, &t->p[tt], x);
    double off[6] = {0, 0, 0, 0, 0, 0};
    if (!t->periodic) ball_rec(t, 0, 0.0, fdist2, off, x, tt, 1, &o);
    else if (t->nodes[0].left < 0) ball_rec(t, 0, 0.0, fdist2, off, x, -1, 1, &o);
    else ball_periodic(t, fdist2, x, 1, &o);
    return o.cnt;
}

int pt_ball_tagged_pos(PTree* t, const double* xq, double fdist2, int* out_ids) {
    BallOut o = {out_ids, 0, NULL, NULL, 0};
    double off[6] = {0, 0, 0, 0, 0, 0};
    if (!t->periodic || t->nodes[0].left < 0) ball_rec(t, 0, 0.0, fdist2, off, xq, -1, 1, &o);
    else ball_periodic(t, fdist2, xq, 1, &o);
    return o.cnt;
}

int pt_ball_mark(PTree* t, int id, double fdist2, int imark, int* mark, double* dist2) {
    BallOut o = {NULL, 0, mark, dist2, imark};
    int tt = t->tree_of_id[id];
    double x[6];
    tvec(t, &t->p[tt], x);
    double off[6] = {0, 0, 0, 0, 0, 0};
    if (!t->periodic) ball_rec(t, 0, 0.0, fdist2, off, x, tt, 0, &o);
    else if (t->nodes[0].left < 0) ball_rec(t, 0, 0.0, fdist2, off, x, -1, 0, &o);
    else ball_periodic(t, fdist2, x, 0, &o);
    return 0;
}

/* ---------------------------------------------------------------- FOF */
typedef struct {
    PTree* t;
    double fdist2;
    int iGroup, nActive;
    int* Group; /* indexed by ID */
    int *Len, *Head, *Tail, *Next, *Fifo;
    short* BucketFlag;
    int iTail;
    /* FOFCriterion */
    int cmp;
    const double* params;
} FofCtx;

static inline void fof_link(FofCtx* c, int target, int i) {
    /* KDLeafNode.cxx:574-582 list splice */
    c->Group[c->t->p[i].id] = c->iGroup;
    c->Fifo[c->iTail++] = i;
    c->Len[c->iGroup]++;
    c->Next[c->Tail[c->Head[target]]] = c->Head[i];
    c->Tail[c->Head[target]] = c->Tail[c->Head[i]];
    c->Head[i] = c->Head[target];
    if (c->iTail == c->nActive) c->iTail = 0;
}

/* SplitNode/LeafNode::FOFSearchBall (KDSplitNode.cxx:921-988, KDLeafNode.cxx:527-589).
   xq is the target's (possibly mirrored) position, vq its velocity. */
static void fof_search(FofCtx* c, int node, double rd, double* off, int target, const double* xq,
                       const double* vq) {
    PTree* t = c->t;
    const PNode* nd = &t->nodes[node];
    int numdim = t->nd;
    double xph[6];
    for (int j = 0; j < 3; j++) xph[j] = xq[j];
    for (int j = 0; j < 3; j++) xph[3 + j] = vq[j];
    /* the reference reads the target through GetPhase (KDNode.h:299, KDSplitNode.cxx:963) */
    const double* xflag = xph;
    if (nd->left < 0) {
        if (c->BucketFlag[node]) return;
        int flag = 1;
        int fl = flag_node(nd, numdim, xflag, c->fdist2);
        if (fl == 1) {
            for (int i = nd->start; i < nd->end; i++) {
                if (c->Group[t->p[i].id]) continue;
                fof_link(c, target, i);
            }
            c->BucketFlag[node] = 1;
        } else {
            for (int i = nd->start; i < nd->end; i++) {
                if (c->Group[t->p[i].id]) continue;
                double d2 = dist2_n(xq, t->p[i].pos, 3);
                if (numdim == 6) d2 += dist2_n(vq, t->p[i].vel, 3);
                if (d2 < c->fdist2) fof_link(c, target, i);
                else flag = 0;
            }
            if (flag) c->BucketFlag[node] = 1;
        }
        return;
    }
    if (c->BucketFlag[node] && c->Head[target] == c->Head[nd->start]) return;
    int fl = flag_node(nd, numdim, xflag, c->fdist2);
    if (fl == 1) {
        for (int i = nd->start; i < nd->end; i++) {
            if (c->Group[t->p[i].id]) continue;
            c->Group[t->p[i].id] = c->iGroup;
            c->Fifo[c->iTail++] = i;
            c->Len[c->iGroup]++;
            c->Next[c->Tail[c->Head[target]]] = c->Head[i];
            c->Tail[c->Head[target]] = c->Tail[c->Head[i]];
            c->Head[i] = c->Head[target];
            c->iTail %= c->nActive;
        }
        c->BucketFlag[node] = 1;
        return;
    }
    int cd = nd->cut_dim;
    double old_off = off[cd];
    double new_off = xflag[cd] - nd->cut_val;
    if (new_off < 0) {
        fof_search(c, nd->left, rd, off, target, xq, vq);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < c->fdist2) {
            off[cd] = new_off;
            fof_search(c, nd->right, rd, off, target, xq, vq);
            off[cd] = old_off;
        }
    } else {
        fof_search(c, nd->right, rd, off, target, xq, vq);
        rd += -old_off * old_off + new_off * new_off;
        if (rd < c->fdist2) {
            off[cd] = new_off;
            fof_search(c, nd->left, rd, off, target, xq, vq);
            off[cd] = old_off;
        }
    }
    if (c->BucketFlag[nd->left] == 1 && c->BucketFlag[nd->right] == 1) c->BucketFlag[node] = 1;
}

/* FOF comparators (FOFFunc.h:30-55) on the target's (possibly mirrored) coordinates. */
static int fof_cmp(const FofCtx* c, const double* xa, const double* va, const PPart* b) {
    const double* params = c->params;
    double total = 0;
    if (c->cmp == 0) {
        for (int j = 0; j < 3; j++) total += (xa[j] - b->pos[j]) * (xa[j] - b->pos[j]) / params[6];
    } else if (c->cmp == 1) {
        for (int j = 0; j < 3; j++) total += (va[j] - b->vel[j]) * (va[j] - b->vel[j]) / params[6];
    } else {
        for (int j = 0; j < 3; j++) {
            total += (xa[j] - b->pos[j]) * (xa[j] - b->pos[j]) / params[6];
            total += (va[j] - b->vel[j]) * (va[j] - b->vel[j]) / params[7];
        }
    }
    return (total < 1);
}

/* SplitNode/LeafNode::FOFSearchCriterion (KDSplitNode.cxx:991-1028, KDLeafNode.cxx:591-619). */
static void fof_search_crit(FofCtx* c, int node, double rd, double* off, int target,
                            const double* xq, const double* vq) {
    PTree* t = c->t;
    const PNode* nd = &t->nodes[node];
    if (c->BucketFlag[node] && c->Head[target] == c->Head[nd->start]) return;
    if (nd->left < 0) {
        int flag = c->Head[nd->start];
        for (int i = nd->start; i < nd->end; i++) {
            if (flag != c->Head[i]) flag = 0;
            int id = t->p[i].id;
            if (c->Group[id] == c->iGroup) continue;
            if (c->Group[id] < 0) continue;
            if (fof_cmp(c, xq, vq, &t->p[i])) {
                fof_link(c, target, i);
                flag = 0;
            }
        }
        if (flag) c->BucketFlag[node] = 1;
        return;
    }
    const double* params = c->params;
    int cd = nd->cut_dim;
    double old_off = off[cd];
    double xph[6] = {xq[0], xq[1], xq[2], vq[0], vq[1], vq[2]};
    double new_off = xph[cd] - nd->cut_val; /* GetPhase, KDSplitNode.cxx:996 */
    double invscaling;
    if ((int)params[0] == TPHYS) invscaling = 1.0 / params[1];
    else if ((int)params[0] == TVEL) invscaling = 1.0 / params[2];
    else if ((int)params[0] == TPHS) invscaling = 1.0 / (params[(cd < 3) * 1 + (cd >= 3) * 2]);
    else invscaling = 1.0;
    if (new_off < 0) {
        fof_search_crit(c, nd->left, rd, off, target, xq, vq);
        rd += (-old_off * old_off + new_off * new_off) * invscaling;
        if (rd < 1) {
            off[cd] = new_off;
            fof_search_crit(c, nd->right, rd, off, target, xq, vq);
            off[cd] = old_off;
        }
    } else {
        fof_search_crit(c, nd->right, rd, off, target, xq, vq);
        rd += (-old_off * old_off + new_off * new_off) * invscaling;
        if (rd < 1) {
            off[cd] = new_off;
            fof_search_crit(c, nd->left, rd, off, target, xq, vq);
            off[cd] = old_off;
        }
    }
    if (c->BucketFlag[nd->left] == 1 && c->BucketFlag[nd->right] == 1) c->BucketFlag[node] = 1;
}

/* The per-member search step of FOF / FOFCriterion, periodic wrappers included
   (KDSplitNode.cxx:1602-1646 gated by fdist2 > sval^2; :1649-1681 ungated). */
static void fof_member(FofCtx* c, int crit, int iid) {
    PTree* t = c->t;
    double off[6] = {0, 0, 0, 0, 0, 0};
    const double* x0 = t->p[iid].pos;
    const double* v0 = t->p[iid].vel;
    int root_leaf = t->nodes[0].left < 0;
    if (crit) fof_search_crit(c, 0, 0.0, off, iid, x0, v0);
    else fof_search(c, 0, 0.0, off, iid, x0, v0);
    if (!t->periodic || root_leaf) return;
    double xp[3];
    for (int m = 0; m < 7; m++) {
        for (int j = 0; j < 6; j++) off[j] = 0.0;
        double sval = reflect(x0, xp, t->period, kImageMask[m]);
        if (crit) fof_search_crit(c, 0, 0.0, off, iid, xp, v0);
        else if (c->fdist2 > sval * sval) fof_search(c, 0, 0.0, off, iid, xp, v0);
    }
}

/* KDTree::FOF / FOFCriterion driver (KDFOF.cxx:29-153, 157-265). Groups are numbered in
   the order their first (tree-order) member is met; groups below minnum are dropped and
   their numbers reused; order=1 renumbers by size through the max-heap. */
static int fof_driver(PTree* t, int crit, double fdist2, int cmp, const double* params,
                      int minnum, int order, int* group, int* ngroup) {
    int n = t->n;
    FofCtx c;
    memset(&c, 0, sizeof(c));
    c.t = t;
    c.fdist2 = fdist2;
    c.nActive = n;
    c.cmp = cmp;
    c.params = params;
    c.Group = group;
    int* pGroupHead = (int*)malloc(sizeof(int) * (n + 1));
    c.Fifo = (int*)malloc(sizeof(int) * n);
    c.BucketFlag = (short*)calloc((size_t)t->numnodes, sizeof(short));
    c.Head = (int*)malloc(sizeof(int) * n);
    c.Next = (int*)malloc(sizeof(int) * n);
    c.Len = (int*)malloc(sizeof(int) * (n + 1));
    c.Tail = (int*)malloc(sizeof(int) * n);
    int iHead = 0;
    c.iTail = 0;
    c.iGroup = 0;
    for (int i = 0; i < n; i++) {
        c.Head[i] = c.Tail[i] = i;
        c.Next[i] = -1;
        group[t->p[i].id] = 0;
    }
    for (int i = 0; i < n; i++) {
        int id = t->p[i].id;
        if (group[id] != 0) continue;
        group[id] = ++c.iGroup;
        c.Len[c.iGroup] = 1;
        pGroupHead[c.iGroup] = i;
        c.Fifo[c.iTail++] = i;
        if (c.iTail == n) c.iTail = 0;
        while (iHead != c.iTail) {
            int iid = c.Fifo[iHead++];
            if (iHead == n) iHead = 0;
            fof_member(&c, crit, iid);
            /* splay (KDFOF.cxx:18-26) */
            if (iHead != c.iTail) {
                int iTail2 = c.iTail - 1;
                if (iTail2 == -1) iTail2 = n - 1;
                int d = c.Fifo[iTail2];
                c.Fifo[iTail2] = c.Fifo[iHead];
                c.Fifo[iHead] = d;
            }
        }
        if (c.Len[c.iGroup] < minnum) {
            int ii = c.Head[pGroupHead[c.iGroup]];
            do {
                group[t->p[ii].id] = -1;
            } while ((ii = c.Next[ii]) != -1);
            c.Len[c.iGroup--] = 0;
        }
    }
    for (int i = 0; i < n; i++)
        if (group[t->p[i].id] == -1) group[t->p[i].id] = 0;
    int ng = c.iGroup;
    if (ng > 0 && order) {
        /* KDFOF.cxx:118-143: heap over group sizes, largest first. */
        int** plist = (int**)malloc(sizeof(int*) * (ng + 1));
        int* pcount = (int*)calloc((size_t)ng + 1, sizeof(int));
        for (int g = 1; g <= ng; g++) plist[g] = (int*)malloc(sizeof(int) * c.Len[g]);
        for (int i = 0; i < n; i++) {
            int gid = group[t->p[i].id];
            if (gid > 0) plist[gid][pcount[gid]++] = i;
        }
        PQ pq;
        pq_init(&pq, ng);
        for (int g = 1; g <= ng; g++) pq_push(&pq, g, c.Len[g]);
        for (int g = 1; g <= ng; g++) {
            int gid = pq_topq(&pq);
            pq_pop(&pq);
            for (int j = 0; j < c.Len[gid]; j++) group[t->p[plist[gid][j]].id] = g;
            free(plist[gid]);
        }
        pq_free(&pq);
        free(plist);
        free(pcount);
    }
    *ngroup = ng;
    free(pGroupHead);
    free(c.Fifo);
    free(c.BucketFlag);
    free(c.Head);
    free(c.Next);
    free(c.Len);
    free(c.Tail);
    return 0;
}

int pt_fof(PTree* t, double ll, int minnum, int order, int* group, int* ngroup) {
    return fof_driver(t, 0, ll * ll, 0, NULL, minnum, order, group, ngroup);
}

int pt_fof_criterion(PTree* t, int cmp, const double* params, int minnum, int order, int* group,
                     int* ngroup) {
    return fof_driver(t, 1, 0.0, cmp, params, minnum, order, group, ngroup);
}

/* ------------------------------------------------------- FOF over given lists */
/* FOF comparators (FOFFunc.h:30-55) between two particles. */
static int nn_cmp(int cmp, const double* params, const PPart* a, const PPart* b) {
    double total = 0;
    if (cmp == 0) {
        for (int j = 0; j < 3; j++) total += (a->pos[j] - b->pos[j]) * (a->pos[j] - b->pos[j]) / params[6];
    } else if (cmp == 1) {
        for (int j = 0; j < 3; j++) total += (a->vel[j] - b->vel[j]) * (a->vel[j] - b->vel[j]) / params[6];
    } else {
        for (int j = 0; j < 3; j++) {
            total += (a->pos[j] - b->pos[j]) * (a->pos[j] - b->pos[j]) / params[6];
            total += (a->vel[j] - b->vel[j]) * (a->vel[j] - b->vel[j]) / params[7];
        }
    }
    return (total < 1);
}

/* KDTree::FOFNNCriterion / FOFNNDistCriterion (KDFOF.cxx:380-640). Groups grow breadth
   first in tree order; each member is tested against its listed neighbours; a neighbour
   already in an older group brings that whole group in (its member list is spliced onto
   the current one); groups below minnum are cleared and the rest numbered by size through
   the max-heap. With values, params[pidx[k]] take values[target] before each target's
   comparisons (the reference's distfunc(numNN, dist2[target])). */
int pt_fof_nn(PTree* t, int cmp, const double* params_in, int numnn, const int* nn,
              const double* values, int npc, const int* pidx, int minnum, int* group,
              int* ngroup) {
    int n = t->n;
    double params[20];
    for (int k = 0; k < 20; k++) params[k] = params_in[k];
    int* head_of = (int*)malloc(sizeof(int) * (size_t)(n + 1)); /* first member of each group */
    int* fifo = (int*)malloc(sizeof(int) * (size_t)n);
    int* phead = (int*)malloc(sizeof(int) * (size_t)n);
    int* ptail = (int*)malloc(sizeof(int) * (size_t)n);
    int* pnext = (int*)malloc(sizeof(int) * (size_t)n);
    int* plen = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    for (int i = 0; i < n; i++) {
        group[i] = 0;
        phead[i] = ptail[i] = i;
        pnext[i] = -1;
    }
    int ig = 0, qh = 0, qt = 0;
    for (int i = 0; i < n; i++) {
        if (group[t->p[i].id] != 0) continue;
        group[t->p[i].id] = ++ig;
        plen[ig] = 1;
        head_of[ig] = i;
        fifo[qt++] = i;
        if (qt == n) qt = 0;
        while (qh != qt) {
            int target = fifo[qh++];
            if (qh == n) qh = 0;
            if (values)
                for (int k = 0; k < npc; k++) params[pidx[k]] = values[target];
            for (int j = 0; j < numnn; j++) {
                int nb = nn[(size_t)target * numnn + j];
                int nid = t->p[nb].id;
                if (group[nid] == ig) continue;
                if (!nn_cmp(cmp, params, &t->p[target], &t->p[nb])) continue;
                if (group[nid] > 0) {
                    int old = group[nid], oh = head_of[old], otail = ptail[oh];
                    int ctail = ptail[head_of[ig]];
                    int m = oh;
                    do {
                        group[t->p[m].id] = ig;
                        phead[m] = head_of[ig];
                    } while ((m = pnext[m]) != -1);
                    m = ctail;
                    do {
                        ptail[m] = otail;
                    } while ((m = pnext[m]) != -1);
                    plen[ig] += plen[old];
                    plen[old] = -1;
                    pnext[ctail] = oh;
                    ptail[head_of[ig]] = otail;
                    phead[oh] = head_of[ig];
                } else {
                    group[nid] = ig;
                    fifo[qt++] = nb;
                    plen[ig]++;
                    pnext[ptail[head_of[ig]]] = nb;
                    ptail[head_of[ig]] = nb;
                    phead[nb] = head_of[ig];
                    if (qt == n) qt = 0;
                }
            }
        }
    }
    /* members of each live group in tree order, then the minnum cut and the size order */
    int** plist = (int**)malloc(sizeof(int*) * (size_t)(ig + 1));
    int* pcount = (int*)calloc((size_t)ig + 1, sizeof(int));
    for (int g = 1; g <= ig; g++) plist[g] = plen[g] > 0 ? (int*)malloc(sizeof(int) * plen[g]) : NULL;
    for (int i = 0; i < n; i++) {
        int gid = group[t->p[i].id];
        if (gid > 0 && plen[gid] > 0) plist[gid][pcount[gid]++] = i;
    }
    int total = ig, live = ig;
    for (int g = 1; g <= total; g++) {
        if (plen[g] < minnum) {
            if (plen[g] > 0)
                for (int j = 0; j < plen[g]; j++) group[t->p[plist[g][j]].id] = 0;
            plen[g] = 0;
            live--;
        }
    }
    if (live) {
        PQ pq;
        pq_init(&pq, live);
        for (int g = 1; g <= total; g++)
            if (plen[g] > 0) pq_push(&pq, g, plen[g]);
        for (int r = 1; r <= live; r++) {
            int gid = pq_topq(&pq), size = (int)pq_top(&pq);
            pq_pop(&pq);
            for (int j = 0; j < size; j++) group[t->p[plist[gid][j]].id] = r;
        }
        pq_free(&pq);
    }
    for (int g = 1; g <= total; g++) free(plist[g]);
    free(plist);
    free(pcount);
    free(head_of);
    free(fifo);
    free(phead);
    free(ptail);
    free(pnext);
    free(plen);
    *ngroup = live;
    return 0;
}

/* ---------------------------------------------------------------- adjoint */
/* Frozen density model shared by the adjoint and the finite-difference check.
   rho_i = sum_{j in N(i)} w_ij m_j + sum_{l : i in N(l)} w_li m_l,
   w_ij  = 0.5 * norm_i * Wsm(q_ij) with q_ij = r_ij / h_i, h_i = 0.5 r_{i,K(i)},
   norm_i = 1/pow(h_i, 3), the same formula as CalcDensity (KDCalcSmoothQuantities.cxx:
   260-286). K(i) (the farthest neighbour) and each pair's table cell are frozen from
   pos0; within a frozen cell Wsm is linear in q. */
static void frozen_setup(const PTree* t, int k, const int* nn, const double* pos0, int* kfar,
                         int* cell) {
    int n = t->n;
    for (int i = 0; i < n; i++) {
        double best = -1;
        int bj = 0;
        for (int j = 0; j < k; j++) {
            const double* a = pos0 + 3 * (size_t)i;
            const double* b = pos0 + 3 * (size_t)nn[(size_t)i * k + j];
            double d2 = dist2_n(a, b, 3);
            if (d2 > best) {
                best = d2;
                bj = j;
            }
        }
        kfar[i] = bj;
        double hi = 0.5 * sqrt(best);
        for (int j = 0; j < k; j++) {
            const double* a = pos0 + 3 * (size_t)i;
            const double* b = pos0 + 3 * (size_t)nn[(size_t)i * k + j];
            double rij = sqrt(dist2_n(a, b, 3));
            cell[(size_t)i * k + j] = (int)(rij / hi * 0.5 * (t->kernres - 1));
        }
    }
}

static inline double table_val(const PTree* t, int c, double q, double delta) {
    return wsm(q, c, t->kernres, delta, t->kernel);
}
static inline double table_slope(const PTree* t, int c, double delta) {
    if (c < t->kernres - 1) return (t->kernel[c + 1] - t->kernel[c]) / delta;
    return 0.0;
}

int pt_density_frozen(PTree* t, int k, const int* nn, const double* pos0, const double* pos,
                      const double* mass, double* rho) {
    int n = t->n;
    int* kfar = (int*)malloc(sizeof(int) * n);
    int* cell = (int*)malloc(sizeof(int) * (size_t)n * k);
    frozen_setup(t, k, nn, pos0, kfar, cell);
    double delta = 2.0 / (double)(t->kernres - 1);
    for (int i = 0; i < n; i++) rho[i] = 0;
    for (int i = 0; i < n; i++) {
        const double* xi = pos + 3 * (size_t)i;
        int kf = nn[(size_t)i * k + kfar[i]];
        double hi = 0.5 * sqrt(dist2_n(xi, pos + 3 * (size_t)kf, 3));
        double norm = 1.0 / pow(hi, 3.0);
        for (int j = 0; j < k; j++) {
            int jj = nn[(size_t)i * k + j];
            double rij = sqrt(dist2_n(xi, pos + 3 * (size_t)jj, 3));
            double w = 0.5 * table_val(t, cell[(size_t)i * k + j], rij / hi, delta) * norm;
            rho[i] += w * mass[jj];
            rho[jj] += w * mass[i];
        }
    }
    free(kfar);
    free(cell);
    return 0;
}

/* ------------------------------------------------------------ SPH smoothing */
/* The densities the smoothing functions divide by: the caller's (densityset = 1) or
   CalcDensity(nsmooth) (KDCalcSmoothQuantities.cxx:408, 493, 561, ...). */
static int sm_density(PTree* t, int nsmooth, const double* rho) {
    if (rho) {
        for (int i = 0; i < t->n; i++) t->p[i].rho = rho[t->p[i].id];
        return 0;
    }
    double* tmp = (double*)malloc(sizeof(double) * (size_t)(t->n > 0 ? t->n : 1));
    int s = pt_density(t, nsmooth, tmp, NULL);
    free(tmp);
    return s;
}

/* Wsm for an index that may pass the end of the table: the reference reads past its table
   there (only CalcVelDensityWithPhysDensity, whose h comes from a squared distance); this
   restatement returns the last entry instead. */
static inline double wsm_end(double r, int i, int size, double delta, const double* x) {
    if (i >= size) return x[size - 1];
    return wsm(r, i, size, delta, x);
}

/* CalcSmoothVel / CalcSmoothVelDisp / CalcSmoothVelSkew / CalcSmoothVelKurtosis
   (KDCalcSmoothQuantities.cxx:480-766): symmetric SPH sums over the Nsmooth nearest. */
int pt_smooth_vel_moments(PTree* t, int which, int nsmooth, const double* rho,
                          const double* smvel, const double* disp, double* out) {
    int n = t->n, nd = t->nd;
    int width = which == 1 ? 9 : 3;
    int status = sm_density(t, nsmooth, rho);
    if (status) return status;
    for (size_t i = 0; i < (size_t)n * width; i++) out[i] = 0;
    PQ pq;
    pq_init(&pq, nsmooth);
    double delta = 2.0 / (double)(t->kernres - 1);
    for (int i = 0; i < n && !status; i++) {
        pq.n = 0;
        for (int j = 0; j < nsmooth; j++) pq_push(&pq, -1, MAXVALUE);
        double off[6] = {0, 0, 0, 0, 0, 0};
        double xt[6] = {0, 0, 0, 0, 0, 0};
        tvec(t, &t->p[i], xt);
        knn_target(t, 0, 0.0, &pq, off, i, xt);
        double hi = 0.5 * sqrt(pq_top(&pq));
        double norm = 1.0 / pow(hi, (double)(nd * 1.));
        for (int j = 0; j < nsmooth; j++) {
            if (pq_topq(&pq) == -1) {
                status = 6;
                break;
            }
            double rij = sqrt(pq_top(&pq));
            double wij = 0.5 * wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres,
                                   delta, t->kernel) *
                         norm;
            int index = pq_topq(&pq);
            int id1 = t->p[i].id, id2 = t->p[index].id;
            const PPart* a = &t->p[index]; /* the neighbour, summed into id1 */
            const PPart* b = &t->p[i];     /* the target, summed into id2 */
            for (int side = 0; side < 2; side++) {
                const PPart* src = side == 0 ? a : b;
                int dst = side == 0 ? id1 : id2;
                double temp = wij / src->rho * src->mass;
                if (which == 0) {
                    for (int k = 0; k < 3; k++) out[(size_t)dst * 3 + k] += temp * src->vel[k];
                } else if (which == 1) {
                    for (int k = 0; k < 3; k++)
                        for (int l = 0; l < 3; l++) {
                            double dv1 = src->vel[k] - smvel[(size_t)dst * 3 + k];
                            double dv2 = src->vel[l] - smvel[(size_t)dst * 3 + l];
                            out[(size_t)dst * 9 + k * 3 + l] += temp * dv1 * dv2;
                        }
                } else if (which == 2) {
                    for (int k = 0; k < 3; k++) {
                        double dv1 = src->vel[k] - smvel[(size_t)dst * 3 + k];
                        out[(size_t)dst * 3 + k] +=
                            temp * dv1 * dv1 * dv1 / pow(disp[(size_t)dst * 9 + k * 4], (double)1.5);
                    }
                } else {
                    for (int k = 0; k < 3; k++) {
                        double dv1 = src->vel[k] - smvel[(size_t)dst * 3 + k];
                        double dkk = disp[(size_t)dst * 9 + k * 4];
                        out[(size_t)dst * 3 + k] += temp * dv1 * dv1 * dv1 * dv1 / (dkk * dkk) - 3.;
                    }
                }
            }
            pq_pop(&pq);
        }
    }
    pq_free(&pq);
    return status;
}

/* CalcVelDensityWithPhysDensity[Particle] (KDCalcSmoothQuantities.cxx:393-478, 922-990):
   the physical h is half the largest squared distance, as the reference computes it. */
static double veldensity_phys_one(PTree* t, int i, int nsmooth, int nsearch, PQ* pq, PQ* pq2,
                                  int* nnids, double* vdist, int* status) {
    int nd = t->nd;
    double delta = 2.0 / (double)(t->kernres - 1);
    pq->n = 0;
    for (int j = 0; j < nsearch; j++) pq_push(pq, -1, MAXVALUE);
    double off[6] = {0, 0, 0, 0, 0, 0};
    double xt[6] = {0, 0, 0, 0, 0, 0};
    tvec(t, &t->p[i], xt);
    knn_target(t, 0, 0.0, pq, off, i, xt);
    double hi = 0.5 * pq_top(pq);
    double norm = 1.0 / pow(hi, (double)(nd * 1.));
    for (int j = 0; j < nsearch; j++) {
        if (pq_topq(pq) == -1) {
            *status = 6;
            return 0;
        }
        nnids[j] = pq_topq(pq);
        vdist[j] = sqrt(dist2_n(t->p[i].vel, t->p[nnids[j]].vel, 3));
        pq_pop(pq);
    }
    pq2->n = 0;
    for (int j = 0; j < nsmooth; j++) pq_push(pq2, -1, MAXVALUE);
    for (int j = 0; j < nsearch; j++)
        if (vdist[j] < pq_top(pq2)) {
            pq_pop(pq2);
            pq_push(pq2, nnids[j], vdist[j]);
        }
    double vhi = 0.5 * pq_top(pq2);
    double vnorm = 1.0 / pow(vhi, (double)(nd * 1.));
    double vden = 0;
    for (int j = 0; j < nsmooth; j++) {
        double vij = pq_top(pq2);
        int id2 = pq_topq(pq2);
        double rij = sqrt(dist2_n(t->p[i].pos, t->p[id2].pos, 3));
        double vwij = wsm_end(vij / vhi, (int)(vij / vhi * 0.5 * (t->kernres - 1)), t->kernres,
                              delta, t->kernel) *
                      vnorm;
        double wij = wsm_end(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres, delta,
                             t->kernel) *
                     norm;
        vden += vwij * (wij / t->p[i].rho * t->p[i].mass);
        pq_pop(pq2);
    }
    return vden;
}

int pt_veldensity_phys(PTree* t, int nsmooth, int nsearch, const double* rho, double* out) {
    if (nsmooth > nsearch) nsmooth = nsearch;
    int status = sm_density(t, nsmooth, rho);
    if (status) return status;
    PQ pq, pq2;
    pq_init(&pq, nsearch);
    pq_init(&pq2, nsmooth);
    int* nnids = (int*)malloc(sizeof(int) * (size_t)nsearch);
    double* vdist = (double*)malloc(sizeof(double) * (size_t)nsearch);
    for (int i = 0; i < t->n; i++) out[i] = 0;
    for (int i = 0; i < t->n && !status; i++)
        out[t->p[i].id] += veldensity_phys_one(t, i, nsmooth, nsearch, &pq, &pq2, nnids, vdist, &status);
    free(nnids);
    free(vdist);
    pq_free(&pq);
    pq_free(&pq2);
    return status;
}

double pt_veldensity_phys_particle(PTree* t, int id, int nsmooth, int nsearch, const double* rho) {
    if (nsmooth > nsearch) nsmooth = nsearch;
    int status = sm_density(t, nsmooth, rho);
    if (status) return NAN;
    PQ pq, pq2;
    pq_init(&pq, nsearch);
    pq_init(&pq2, nsmooth);
    int* nnids = (int*)malloc(sizeof(int) * (size_t)nsearch);
    double* vdist = (double*)malloc(sizeof(double) * (size_t)nsearch);
    double v = veldensity_phys_one(t, t->tree_of_id[id], nsmooth, nsearch, &pq, &pq2, nnids, vdist,
                                   &status);
    free(nnids);
    free(vdist);
    pq_free(&pq);
    pq_free(&pq2);
    return status ? NAN : v;
}

/* CalcSmoothVel{Particle,Position}, CalcSmoothVelDisp{Particle,Position},
   CalcSmoothLocalMean{Particle,Position}, CalcSmoothLocalDisp{Particle,Position}
   (KDCalcSmoothQuantities.cxx:992-1091, 1209-1306, 1539-1700): one-sided sums. */
int pt_smooth_one(PTree* t, int which, int id, const double* x, int nsmooth, const double* rho,
                  const double* smvel, const double* weight, double mean, double* out) {
    int nd = t->nd;
    int status = sm_density(t, nsmooth, rho);
    if (status) return status;
    int width = which == 1 ? 9 : (which == 0 ? 3 : 1);
    for (int k = 0; k < width; k++) out[k] = 0;
    PQ pq;
    pq_init(&pq, nsmooth);
    for (int j = 0; j < nsmooth; j++) pq_push(&pq, -1, MAXVALUE);
    double off[6] = {0, 0, 0, 0, 0, 0};
    if (x) {
        double xq[6] = {0, 0, 0, 0, 0, 0};
        for (int j = 0; j < nd; j++) xq[j] = x[j];
        knn_coord(t, 0, 0.0, &pq, off, xq);
    } else {
        int i = t->tree_of_id[id];
        double xt[6] = {0, 0, 0, 0, 0, 0};
        tvec(t, &t->p[i], xt);
        knn_target(t, 0, 0.0, &pq, off, i, xt);
    }
    double delta = 2.0 / (double)(t->kernres - 1);
    double hi = 0.5 * sqrt(pq_top(&pq));
    double norm = 1.0 / pow(hi, (double)(nd * 1.));
    for (int j = 0; j < nsmooth; j++) {
        if (pq_topq(&pq) == -1) {
            status = 6;
            break;
        }
        double rij = sqrt(pq_top(&pq));
        double wij = wsm(rij / hi, (int)(rij / hi * 0.5 * (t->kernres - 1)), t->kernres, delta,
                         t->kernel) *
                     norm;
        const PPart* a = &t->p[pq_topq(&pq)];
        double temp = wij / a->rho * a->mass;
        if (which == 0) {
            for (int k = 0; k < 3; k++) out[k] += temp * a->vel[k];
        } else if (which == 1) {
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) {
                    double dv1 = a->vel[k] - smvel[k];
                    double dv2 = a->vel[l] - smvel[l];
                    out[k * 3 + l] += temp * dv1 * dv2;
                }
        } else if (which == 4) {
            out[0] += temp * weight[a->id];
        } else {
            double dl = (weight[a->id] - mean);
            out[0] += temp * dl * dl;
        }
        pq_pop(&pq);
    }
    pq_free(&pq);
    return status;
}

int pt_density_adjoint(PTree* t, int k, const int* nn, const double* pos, const double* mass,
                       const double* wts, double* rho, double* gpos, double* gmass) {
    int n = t->n;
    int* kfar = (int*)malloc(sizeof(int) * n);
    int* cell = (int*)malloc(sizeof(int) * (size_t)n * k);
    frozen_setup(t, k, nn, pos, kfar, cell);
    pt_density_frozen(t, k, nn, pos, pos, mass, rho);
    double delta = 2.0 / (double)(t->kernres - 1);
    double* g = (double*)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) g[i] = wts[i] / rho[i];
    memset(gpos, 0, sizeof(double) * 3 * (size_t)n);
    memset(gmass, 0, sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) {
        const double* xi = pos + 3 * (size_t)i;
        int kf = nn[(size_t)i * k + kfar[i]];
        double rk = sqrt(dist2_n(xi, pos + 3 * (size_t)kf, 3));
        double hi = 0.5 * rk;
        double norm = 1.0 / pow(hi, 3.0);
        double A = 0; /* dL/dh_i */
        for (int j = 0; j < k; j++) {
            int jj = nn[(size_t)i * k + j];
            const double* xj = pos + 3 * (size_t)jj;
            double rij = sqrt(dist2_n(xi, xj, 3));
            double q = rij / hi;
            int c = cell[(size_t)i * k + j];
            double T = table_val(t, c, q, delta);
            double Tp = table_slope(t, c, delta);
            double w = 0.5 * T * norm;
            double cij = g[i] * mass[jj] + g[jj] * mass[i];
            gmass[jj] += g[i] * w;
            gmass[i] += g[jj] * w;
            double dw_dr = 0.5 * norm * Tp / hi;
            double dw_dh = -0.5 * norm / hi * (3.0 * T + q * Tp);
            A += cij * dw_dh;
            double coef = cij * dw_dr / rij;
            for (int d = 0; d < 3; d++) {
                double gd = coef * (xi[d] - xj[d]);
                gpos[3 * (size_t)i + d] += gd;
                gpos[3 * (size_t)jj + d] -= gd;
            }
        }
        double coefh = A * 0.5 / rk;
        const double* xk = pos + 3 * (size_t)kf;
        for (int d = 0; d < 3; d++) {
            double gd = coefh * (xi[d] - xk[d]);
            gpos[3 * (size_t)i + d] += gd;
            gpos[3 * (size_t)kf + d] -= gd;
        }
    }
    free(g);
    free(kfar);
    free(cell);
    return 0;
}

/* ---------------------------------------------------------------- local finite differences */
/* Central finite difference of L = sum_i w_i log rho_i with respect to one coordinate,
   restricted to the loss terms that coordinate can change, on the frozen model above.
   Moving particle a changes w_aj (j in N(a)), w_la (a in N(l)) and h_l for every l whose
   farthest neighbour is a; the affected densities are those of a, N(a), the l's, and
   N(l) for those l. Differencing only these terms avoids the cancellation of a sum over
   every particle. */
typedef struct {
    PTree* t;
    int n, k;
    const int* nn;
    double* pos;
    const double* mass;
    const double* w;
    int* kfar;
    int* cell;
    int *rev_off, *rev_l, *rev_s; /* (l, slot) pairs with nn[l][slot] = i */
    int *kf_off, *kf_l;           /* l with farthest neighbour = i */
    int* mark;
    int* list;
} AdjCtx;

void* pt_adj_create(PTree* t, int k, const int* nn, const double* pos0, const double* mass,
                    const double* w) {
    int n = t->n;
    AdjCtx* c = (AdjCtx*)calloc(1, sizeof(AdjCtx));
    c->t = t;
    c->n = n;
    c->k = k;
    c->nn = nn;
    c->mass = mass;
    c->w = w;
    c->pos = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    memcpy(c->pos, pos0, sizeof(double) * 3 * (size_t)n);
    c->kfar = (int*)malloc(sizeof(int) * n);
    c->cell = (int*)malloc(sizeof(int) * (size_t)n * k);
    frozen_setup(t, k, nn, pos0, c->kfar, c->cell);
    c->rev_off = (int*)calloc((size_t)n + 1, sizeof(int));
    c->kf_off = (int*)calloc((size_t)n + 1, sizeof(int));
    for (size_t e = 0; e < (size_t)n * k; e++) c->rev_off[nn[e] + 1]++;
    for (int i = 0; i < n; i++) c->kf_off[nn[(size_t)i * k + c->kfar[i]] + 1]++;
    for (int i = 0; i < n; i++) {
        c->rev_off[i + 1] += c->rev_off[i];
        c->kf_off[i + 1] += c->kf_off[i];
    }
    c->rev_l = (int*)malloc(sizeof(int) * (size_t)n * k);
    c->rev_s = (int*)malloc(sizeof(int) * (size_t)n * k);
    c->kf_l = (int*)malloc(sizeof(int) * n);
    int* fill = (int*)calloc((size_t)n, sizeof(int));
    for (int l = 0; l < n; l++)
        for (int s = 0; s < k; s++) {
            int i = nn[(size_t)l * k + s];
            int p = c->rev_off[i] + fill[i]++;
            c->rev_l[p] = l;
            c->rev_s[p] = s;
        }
    memset(fill, 0, sizeof(int) * n);
    for (int l = 0; l < n; l++) {
        int a = nn[(size_t)l * k + c->kfar[l]];
        c->kf_l[c->kf_off[a] + fill[a]++] = l;
    }
    free(fill);
    c->mark = (int*)calloc((size_t)n, sizeof(int));
    c->list = (int*)malloc(sizeof(int) * (size_t)n);
    return c;
}

void pt_adj_destroy(void* h) {
    AdjCtx* c = (AdjCtx*)h;
    if (!c) return;
    free(c->pos);
    free(c->kfar);
    free(c->cell);
    free(c->rev_off);
    free(c->rev_l);
    free(c->rev_s);
    free(c->kf_off);
    free(c->kf_l);
    free(c->mark);
    free(c->list);
    free(c);
}

static double adj_h(const AdjCtx* c, int l) {
    const double* xl = c->pos + 3 * (size_t)l;
    int kf = c->nn[(size_t)l * c->k + c->kfar[l]];
    return 0.5 * sqrt(dist2_n(xl, c->pos + 3 * (size_t)kf, 3));
}

static double adj_w(const AdjCtx* c, int l, int s, double hl) {
    int j = c->nn[(size_t)l * c->k + s];
    double r = sqrt(dist2_n(c->pos + 3 * (size_t)l, c->pos + 3 * (size_t)j, 3));
    double delta = 2.0 / (double)(c->t->kernres - 1);
    double T = table_val(c->t, c->cell[(size_t)l * c->k + s], r / hl, delta);
    return 0.5 * T / pow(hl, 3.0);
}

static double adj_rho(const AdjCtx* c, int i) {
    double rho = 0, hi = adj_h(c, i);
    for (int s = 0; s < c->k; s++) rho += adj_w(c, i, s, hi) * c->mass[c->nn[(size_t)i * c->k + s]];
    for (int p = c->rev_off[i]; p < c->rev_off[i + 1]; p++) {
        int l = c->rev_l[p];
        rho += adj_w(c, l, c->rev_s[p], adj_h(c, l)) * c->mass[l];
    }
    return rho;
}

double pt_adj_fd(void* h, int a, int d, double step) {
    AdjCtx* c = (AdjCtx*)h;
    int cnt = 0;
#define ADD(x)                         \
    do {                               \
        int _x = (x);                  \
        if (!c->mark[_x]) {            \
            c->mark[_x] = 1;           \
            c->list[cnt++] = _x;       \
        }                              \
    } while (0)
    ADD(a);
    for (int s = 0; s < c->k; s++) ADD(c->nn[(size_t)a * c->k + s]);
    for (int p = c->rev_off[a]; p < c->rev_off[a + 1]; p++) ADD(c->rev_l[p]);
    for (int p = c->kf_off[a]; p < c->kf_off[a + 1]; p++) {
        int l = c->kf_l[p];
        ADD(l);
        for (int s = 0; s < c->k; s++) ADD(c->nn[(size_t)l * c->k + s]);
    }
#undef ADD
    double x0 = c->pos[3 * (size_t)a + d];
    double sum = 0;
    double* rp = (double*)malloc(sizeof(double) * cnt);
    c->pos[3 * (size_t)a + d] = x0 + step;
    for (int q = 0; q < cnt; q++) rp[q] = adj_rho(c, c->list[q]);
    c->pos[3 * (size_t)a + d] = x0 - step;
    for (int q = 0; q < cnt; q++) {
        double rm = adj_rho(c, c->list[q]);
        sum += c->w[c->list[q]] * log1p((rp[q] - rm) / rm);
    }
    c->pos[3 * (size_t)a + d] = x0;
    for (int q = 0; q < cnt; q++) c->mark[c->list[q]] = 0;
    free(rp);
    return sum / (2 * step);
}
