/*
 * Test infrastructure only. C restatement of the reference NBodylib KDTree hot path
 * (src/KDTree/), used as the CPU checker by tests/ and as the CPU baseline by bench.py.
 * It is never linked into the product library. Parity of this restatement is pinned
 * against the reference itself (oracle/_ref/libnbref.so) by tests/test_oracle.py
 * and against the committed golden fixtures in tests/golden/.
 *
 * Indices: every neighbour list and every per-particle output is in input order ("ID"
 * in the reference, set to the input index at KDTree.cxx:1291).
 */
#ifndef NBPORT_H
#define NBPORT_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct PTree PTree;

/* treetype: 0 physical (TPHYS), 2 velocity (TVEL), 3 phase space (TPHS).
   kerntype: 0 M4 spline (KSPH), 1 Gaussian, 2 Epanechnikov, 3 top-hat. period may be NULL. */
PTree* pt_create(const double* pos, const double* vel, const double* mass, int n, int b,
                 int treetype, int kerntype, int kernres, const double* period, int nthreads);
void pt_destroy(PTree* t);
/* The reference's Aniso constructor argument for phase-space trees: -1 plain phase-space
   distance (FindNearestPhase), 0 local metric (CalculateMetricSpacing + FindNearestMetric,
   the reference's default). */
void pt_set_aniso(PTree* t, int aniso);
int pt_num_nodes(const PTree* t);
int pt_num_leaves(const PTree* t);
double pt_kernnorm(const PTree* t);
void pt_kernel_table(const PTree* t, double* table);
void pt_ids(const PTree* t, int* ids);
void pt_leaf_start(const PTree* t, int* leaf_start);
double pt_build_seconds(const PTree* t);

/* method 0: FindNearest(tt), 1: FindNearestPos(tt) (physical trees). Row i belongs to the
   particle with ID i. Returns 6 when a phase-space metric spacing fails, 7 if unsupported. */
int pt_knn(PTree* t, int method, int k, int nthreads, int* nn_ids, double* d2);
/* FindNearestPos(x) for nq coordinates. */
int pt_knn_pos(PTree* t, const double* x, int nq, int k, int nthreads, int* nn_ids, double* d2);
/* FindNearest(x) for nq coordinates of the tree's space (3 or 6 per row). */
int pt_knn_coord(PTree* t, const double* x, int nq, int k, int nthreads, int* nn_ids, double* d2);
/* CalcDensity(k) (KDCalcSmoothQuantities.cxx:203-305). rho in ID order. If nn_ids is not
   NULL it receives the k neighbours of each particle (ID rows, descending d2 as the heap
   pops them) so that tests can freeze them for the adjoint. */
int pt_density(PTree* t, int k, double* rho, int* nn_ids);
int pt_veldensity(PTree* t, int nsmooth, int nsearch, double* out);
/* The same two over OpenMP threads (physical and velocity trees): the parallel density
   sums each particle's terms in another order (within a few ulps of pt_density); the
   velocity density is bit-identical to pt_veldensity. Status 7 for phase-space trees. */
int pt_density_parallel(PTree* t, int k, int nthreads, double* rho);
int pt_veldensity_parallel(PTree* t, int nsmooth, int nsearch, int nthreads, double* out);
double pt_density_particle(PTree* t, int id, int k);
double pt_veldensity_particle(PTree* t, int id, int nsmooth, int nsearch);
double pt_density_position(PTree* t, const double* x, int k);
double pt_veldensity_position(PTree* t, const double* x, const double* v, int nsmooth,
                              int nsearch);
int pt_fof(PTree* t, double ll, int minnum, int order, int* group, int* ngroup);
/* cmp: 0 FOF3d, 1 FOFVel, 2 FOF6d (src/KDTree/FOFFunc.h:30-55). params as the reference. */
int pt_fof_criterion(PTree* t, int cmp, const double* params, int minnum, int order, int* group,
                     int* ngroup);
/* FOFNNCriterion / FOFNNDistCriterion over lists nn (rows by tree index, tree indices);
   values (tree order) with npc parameter indices pidx, or NULL. group in ID order. */
int pt_fof_nn(PTree* t, int cmp, const double* params, int numnn, const int* nn,
              const double* values, int npc, const int* pidx, int minnum, int* group,
              int* ngroup);
int pt_ball_tagged(PTree* t, int id, double fdist2, int* out_ids);
int pt_ball_tagged_pos(PTree* t, const double* x, double fdist2, int* out_ids);
int pt_ball_mark(PTree* t, int id, double fdist2, int imark, int* mark, double* dist2);

/* SPH smoothing over the Nsmooth nearest neighbours (KDCalcSmoothQuantities.cxx).
   rho: the particles' densities in ID order (the reference's densityset = 1), or NULL to
   run CalcDensity(nsmooth) first (densityset != 1). Outputs in ID order.
   which: 0 CalcSmoothVel (out n*3), 1 CalcSmoothVelDisp (n*9, row-major (k,l); needs
   smvel n*3), 2 CalcSmoothVelSkew (n*3; needs smvel, disp), 3 CalcSmoothVelKurtosis. */
int pt_smooth_vel_moments(PTree* t, int which, int nsmooth, const double* rho,
                          const double* smvel, const double* disp, double* out);
/* CalcVelDensityWithPhysDensity (all particles, ID order) and its Particle form. */
int pt_veldensity_phys(PTree* t, int nsmooth, int nsearch, const double* rho, double* out);
double pt_veldensity_phys_particle(PTree* t, int id, int nsmooth, int nsearch, const double* rho);
/* Single-particle (x == NULL, target id) and position (x) forms:
   which 0 CalcSmoothVel{Particle,Position} (out 3), 1 CalcSmoothVelDisp{..} (out 9, needs
   smvel 3), 4 CalcSmoothLocalMean{..} (out 1, needs weight in ID order),
   5 CalcSmoothLocalDisp{..} (out 1, needs weight and mean). */
int pt_smooth_one(PTree* t, int which, int id, const double* x, int nsmooth, const double* rho,
                  const double* smvel, const double* weight, double mean, double* out);

/* Density adjoint (no reference counterpart): L = sum_i w_i log rho_i with rho from
   CalcDensity(k), neighbour lists nn_ids (ID rows of k, any order) and kernel-table cells
   frozen. Inputs/outputs in ID order; pos is (n,3) row-major. */
int pt_density_adjoint(PTree* t, int k, const int* nn_ids, const double* pos,
                       const double* mass, const double* w, double* rho_out,
                       double* grad_pos, double* grad_mass);
/* Density from frozen neighbour lists and frozen table cells (cells taken from pos0),
   evaluated at positions pos; used by the finite-difference check. */
int pt_density_frozen(PTree* t, int k, const int* nn_ids, const double* pos0,
                      const double* pos, const double* mass, double* rho_out);
/* Central finite difference dL/dpos[a][d] of the frozen model, differencing only the
   loss terms that coordinate changes. The context keeps pointers to nn_ids, mass, w. */
void* pt_adj_create(PTree* t, int k, const int* nn_ids, const double* pos0,
                    const double* mass, const double* w);
double pt_adj_fd(void* ctx, int a, int d, double step);
void pt_adj_destroy(void* ctx);

#ifdef __cplusplus
}
#endif
#endif
