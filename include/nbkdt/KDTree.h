/*
 * nbkdt/KDTree.h -- source-compatible drop-in for NBodylib's NBody::KDTree
 * (src/KDTree/KDTree.h) over the GB300 C ABI (include/nbkdt.h, libnbkdt.so).
 *
 * Include this header instead of the reference's KDTree.h and link libnbkdt.so instead
 * of the reference's KDTree library; the caller's NBody::Particle / NBody::System come
 * from NBodylib's NBody.h as before. The constructors and the hot-path methods keep the
 * reference's signatures and meaning:
 *  - the constructor reorders the caller's particle array into the tree's leaf order and
 *    sets each particle's ID to its input index (KDTree.h:12-15, KDTree.cxx:1291); the
 *    destructor restores the input order by sorting on ID (KDTree.cxx:1340-1356);
 *  - neighbour lists hold tree indices into that array (KDTree.h:295); ID-indexed
 *    outputs (FOF groups, SearchBallPos marks, densities) are ID-indexed as before.
 * Differences: errors the reference answers with printf + exit(1) throw
 * nbkdt::Error instead; options the GPU path does not run (a splitting criterion other
 * than 0, anisotropic or scaled metrics, adaptive trees, tree types other than TPHYS, a
 * FOF comparator other than FOF3d / FOFVel / FOF6d) throw nbkdt::Error with status
 * NBK_ERR_UNSUPPORTED. The tree's leaves hold the same particles as the reference's,
 * but their order inside a leaf differs, so tree indices differ; compare results by ID.
 */
#ifndef NBKDT_KDTREE_H
#define NBKDT_KDTREE_H

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <NBody.h>

#include "../nbkdt.h"

namespace nbkdt {
class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& msg) : std::runtime_error(msg), status(status) {}
  int status;
};
inline void check(int status) {
  if (status != NBK_OK) throw Error(status, nbk_last_error());
}
}  // namespace nbkdt

namespace NBody {

// FOF comparator types and the comparators the GPU path recognises (FOFFunc.h:24-57):
// link when the summed squared separations, each divided by its linking length^2, are
// below 1.
typedef int (*FOFcompfunc)(Particle&, Particle&, Double_t*);
typedef int (*FOFcheckfunc)(Particle&, Double_t*);
inline int FOF3d(Particle& a, Particle& b, Double_t* params) {
  Double_t total = 0;
  for (int j = 0; j < 3; j++)
    total += (a.GetPosition(j) - b.GetPosition(j)) * (a.GetPosition(j) - b.GetPosition(j)) / params[6];
  return total < 1;
}
inline int FOFVel(Particle& a, Particle& b, Double_t* params) {
  Double_t total = 0;
  for (int j = 0; j < 3; j++)
    total += (a.GetVelocity(j) - b.GetVelocity(j)) * (a.GetVelocity(j) - b.GetVelocity(j)) / params[6];
  return total < 1;
}
inline int FOF6d(Particle& a, Particle& b, Double_t* params) {
  Double_t total = 0;
  for (int j = 0; j < 3; j++) {
    total += (a.GetPosition(j) - b.GetPosition(j)) * (a.GetPosition(j) - b.GetPosition(j)) / params[6];
    total += (a.GetVelocity(j) - b.GetVelocity(j)) * (a.GetVelocity(j) - b.GetVelocity(j)) / params[7];
  }
  return total < 1;
}
inline int Pnocheck(Particle&, Double_t*) { return 0; }

class KDTree {
 public:
  const static int TPHYS = 0, TPROJ = 1, TVEL = 2, TPHS = 3, TMETRIC = 4;
  const static int KSPH = 0, KGAUSS = 1, KEPAN = 2, KTH = 3;
  const static int KDTREE_SPLIT_ENTROPY = 1, KDTREE_SPLIT_DISPERSION = 2,
                   KDTREE_SPLIT_MAXINTERPARTICLESPACING = 3, KDTREE_SPLIT_SPREAD = 0;

  // KDTree.h:229-245
  KDTree(Particle* p, Int_t numparts, Int_t bucket_size = 16, int TreeType = TPHYS,
         int KernType = KEPAN, int KernRes = 1000, int SplittingCriterion = KDTREE_SPLIT_SPREAD,
         int Aniso = 0, int ScaleSpace = 0, Double_t* Period = NULL, Double_t** metric = NULL,
         bool iBuildInParallel = true, bool iKeepInputOrder = false, Double_t Rdistadapt = -1,
         Double_t AdaptiveMedianFac = 0.0, Int_t min_bucket_size = 16) {
    (void)iBuildInParallel;
    (void)min_bucket_size;
    init(p, numparts, bucket_size, TreeType, KernType, KernRes, SplittingCriterion, Aniso,
         ScaleSpace, Period, metric, iKeepInputOrder, Rdistadapt, AdaptiveMedianFac);
  }
  // KDTree.h:248-263
  KDTree(std::vector<Particle>& p, Int_t bucket_size = 16, int TreeType = TPHYS,
         int KernType = KEPAN, int KernRes = 1000, int SplittingCriterion = KDTREE_SPLIT_SPREAD,
         int Aniso = 0, int ScaleSpace = 0, Double_t* Period = NULL, Double_t** metric = NULL,
         bool iBuildInParallel = true, bool iKeepInputOrder = false, Double_t Rdistadapt = -1,
         Double_t AdaptiveMedianFac = 0.0, Int_t min_bucket_size = 16)
      : KDTree(p.data(), (Int_t)p.size(), bucket_size, TreeType, KernType, KernRes,
               SplittingCriterion, Aniso, ScaleSpace, Period, metric, iBuildInParallel,
               iKeepInputOrder, Rdistadapt, AdaptiveMedianFac, min_bucket_size) {}
  // KDTree.h:266-274 (a System whose period is all zero builds a non-periodic tree,
  // KDTree.cxx:1334-1337)
  KDTree(System& s, Int_t bucket_size = 16, int TreeType = TPHYS, int KernType = KEPAN,
         int KernRes = 1000, int SplittingCriterion = 0, int Aniso = 0, int ScaleSpace = 0,
         Double_t** metric = NULL, bool iBuildInParallel = true, bool iKeepInputOrder = false,
         Double_t Rdistadapt = -1, Double_t AdaptiveMedianFac = 0.0, Int_t min_bucket_size = 16) {
    (void)iBuildInParallel;
    (void)min_bucket_size;
    Double_t per[3];
    bool periodic = false;
    for (int j = 0; j < 3; j++) {
      per[j] = s.GetPeriod()[j];
      periodic = periodic || per[j] != 0;
    }
    init(s.Parts(), s.GetNumParts(), bucket_size, TreeType, KernType, KernRes,
         SplittingCriterion, Aniso, ScaleSpace, periodic ? per : NULL, metric, iKeepInputOrder,
         Rdistadapt, AdaptiveMedianFac);
  }
  // KDTree.cxx:1340-1356: put the particles back in input order
  ~KDTree() {
    if (tree_) nbk_destroy(tree_);
    if (iresetorder_)
      std::sort(bucket_, bucket_ + numparts_,
                [](const Particle& a, const Particle& b) { return a.GetID() < b.GetID(); });
  }
  KDTree(const KDTree&) = delete;
  KDTree& operator=(const KDTree&) = delete;

  // KDTree.h:282-289
  Int_t GetNumNodes() { return (Int_t)numnodes_; }
  Int_t GetNumLeafNodes() { return (Int_t)numleaves_; }
  Int_t GetBucketSize() { return b_; }
  Int_t GetTreeType() { return treetype_; }
  Int_t GetKernType() { return kerntype_; }
  Double_t GetKernNorm() { return kernnorm_; }
  Double_t GetPeriod(int j) { return period_[j]; }

  // ---- kNN (KDTree.h:300-313)
  void FindNearest(Int_t tt, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    knn_one(tt, nn, dist2, Nsearch, NBK_FINDNEAREST);
  }
  void FindNearestPos(Int_t tt, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    knn_one(tt, nn, dist2, Nsearch, NBK_FINDNEARESTPOS);
  }
  void FindNearest(Int_t** nn, Double_t** dist2, Int_t Nsearch = 64) {
    knn_all(nn, dist2, Nsearch, NBK_FINDNEAREST);
  }
  void FindNearestPos(Int_t** nn, Double_t** dist2, Int_t Nsearch = 64) {
    knn_all(nn, dist2, Nsearch, NBK_FINDNEARESTPOS);
  }
  // x in the tree's space: x, y, z (physical), vx, vy, vz (velocity) or all six (phase)
  void FindNearest(Double_t* x, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    std::vector<int32_t> n32(Nsearch);
    nbkdt::check(nbk_knn_coords(tree_, x, 1, Nsearch, n32.data(), dist2));
    for (Int_t j = 0; j < Nsearch; j++) nn[j] = n32[j];
  }
  void FindNearestPos(Double_t* x, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    std::vector<int32_t> n32(Nsearch);
    nbkdt::check(nbk_knn_points(tree_, x, 1, Nsearch, NBK_PERIODIC_REF, n32.data(), dist2));
    for (Int_t j = 0; j < Nsearch; j++) nn[j] = n32[j];
  }
  void FindNearestPos(Coordinate x, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    FindNearestPos(x.GetCoord(), nn, dist2, Nsearch);
  }
  // velocity trees: FindNearestVel (KDFindNearest.cxx:335-346, 451-453, 530-541)
  void FindNearestVel(Int_t tt, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    knn_one(tt, nn, dist2, Nsearch, NBK_FINDNEARESTVEL);
  }
  void FindNearestVel(Int_t** nn, Double_t** dist2, Int_t Nsearch = 64) {
    knn_all(nn, dist2, Nsearch, NBK_FINDNEARESTVEL);
  }
  void FindNearestVel(Double_t* v, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    if (treetype_ != TVEL)
      throw nbkdt::Error(NBK_ERR_UNSUPPORTED, "FindNearestVel(v) runs on velocity trees only");
    FindNearest(v, nn, dist2, Nsearch);
  }
  // phase-space trees: FindNearestPhase, the plain phase distance whatever Aniso
  // (KDFindNearest.cxx:347-361, 454-456, 542-560)
  void FindNearestPhase(Int_t tt, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    knn_one(tt, nn, dist2, Nsearch, NBK_FINDNEARESTPHASE);
  }
  void FindNearestPhase(Int_t** nn, Double_t** dist2, Int_t Nsearch = 64) {
    knn_all(nn, dist2, Nsearch, NBK_FINDNEARESTPHASE);
  }
  void FindNearestPhase(Double_t* x, Double_t* v, Int_t* nn, Double_t* dist2, Int_t Nsearch = 64) {
    Double_t xv[6] = {x[0], x[1], x[2], v[0], v[1], v[2]};
    std::vector<int32_t> n32(Nsearch);
    nbkdt::check(nbk_knn_phase_points(tree_, xv, 1, Nsearch, n32.data(), dist2));
    for (Int_t j = 0; j < Nsearch; j++) nn[j] = n32[j];
  }

  // ---- ball search (KDTree.h:341-373)
  void SearchBallPos(Int_t tt, Double_t fdist2, Int_t imark, Int_t* nn, Double_t* dist2) {
    std::vector<int32_t> m(nn, nn + numparts_);
    nbkdt::check(nbk_ball_mark(tree_, (int32_t)tt, fdist2, (int32_t)imark, m.data(), dist2));
    std::copy(m.begin(), m.end(), nn);
  }
  Int_t SearchBallPosTagged(Int_t tt, Double_t fdist2, Int_t* tagged) {
    std::vector<Int_t> v = SearchBallPosTagged(tt, fdist2);
    std::copy(v.begin(), v.end(), tagged);
    return (Int_t)v.size();
  }
  std::vector<Int_t> SearchBallPosTagged(Int_t tt, Double_t fdist2) {
    int32_t t = (int32_t)tt;
    return ball(&t, nullptr, fdist2);
  }
  std::vector<Int_t> SearchBallPosTagged(Double_t* x, Double_t fdist2) {
    return ball(nullptr, x, fdist2);
  }
  std::vector<Int_t> SearchBallPosTagged(Coordinate x, Double_t fdist2) {
    return ball(nullptr, x.GetCoord(), fdist2);
  }
  Int_t SearchBallPosTagged(Double_t* x, Double_t fdist2, Int_t* tagged) {
    std::vector<Int_t> v = ball(nullptr, x, fdist2);
    std::copy(v.begin(), v.end(), tagged);
    return (Int_t)v.size();
  }

  // ---- SPH (KDTree.h:407-425); results land in Particle::rho, as the reference's do
  void CalcDensity(Int_t Nsmooth = 64) {
    std::vector<double> rho(numparts_);
    nbkdt::check(nbk_density(tree_, Nsmooth, rho.data()));
    for (Int_t i = 0; i < numparts_; i++) bucket_[i].SetDensity(rho[bucket_[i].GetID()]);
  }
  void CalcVelDensity(Int_t Nsmooth = 64, Int_t Nsearch = 64) {
    std::vector<double> v(numparts_);
    nbkdt::check(nbk_veldensity(tree_, Nsmooth, Nsearch, v.data()));
    for (Int_t i = 0; i < numparts_; i++) bucket_[i].SetDensity(v[bucket_[i].GetID()]);
  }
  Double_t CalcDensityParticle(Int_t target, Int_t Nsmooth = 64) {
    int32_t t = (int32_t)target;
    double out = 0;
    nbkdt::check(nbk_density_particles(tree_, &t, 1, Nsmooth, &out));
    return out;
  }
  Double_t CalcVelDensityParticle(Int_t target, Int_t Nsmooth = 64, Int_t Nsearch = 64) {
    int32_t t = (int32_t)target;
    double out = 0;
    nbkdt::check(nbk_veldensity_particles(tree_, &t, 1, Nsmooth, Nsearch, &out));
    return out;
  }
  // CalcDensityPosition / CalcVelDensityPosition (KDTree.h:432-438), physical trees; the
  // velocity argument of CalcDensityPosition only matters for phase-space trees.
  Double_t CalcDensityPosition(Double_t* x, Int_t Nsmooth = 64, Double_t* v = NULL) {
    (void)v;
    double out = 0;
    nbkdt::check(nbk_density_points(tree_, x, 1, Nsmooth, &out));
    return out;
  }
  Double_t CalcDensityPosition(Coordinate x, Int_t Nsmooth = 64, Coordinate v = Coordinate(0.)) {
    return CalcDensityPosition(x.GetCoord(), Nsmooth, v.GetCoord());
  }
  Double_t CalcVelDensityPosition(Double_t* x, Double_t* v, Int_t Nsmooth = 64,
                                  Int_t Nsearch = 64) {
    double out = 0;
    nbkdt::check(nbk_veldensity_points(tree_, x, v, 1, Nsmooth, Nsearch, &out));
    return out;
  }
  Double_t CalcVelDensityPosition(Coordinate x, Coordinate v, Int_t Nsmooth = 64,
                                  Int_t Nsearch = 64) {
    return CalcVelDensityPosition(x.GetCoord(), v.GetCoord(), Nsmooth, Nsearch);
  }

  // ---- SPH smoothing (KDTree.h:413-464, KDCalcSmoothQuantities.cxx). densityset == 1 uses
  // the densities stored in the particles (by CalcDensity), as the reference does; any
  // other value computes CalcDensity(Nsmooth) first. Arrays returned with new[] are indexed
  // by ID, as the reference's. With meanvelset / veldispset != 1 the mean velocities /
  // dispersions are computed here; unlike the reference, the caller's arrays are not deleted.
  Double_t* CalcVelDensityWithPhysDensity(Int_t Nsmooth = 64, Int_t Nsearch = 64,
                                          int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    Double_t* out = new Double_t[numparts_];
    nbkdt::check(nbk_veldensity_physdensity(tree_, Nsmooth, Nsearch, rho_or_null(rho), out));
    return out;
  }
  Coordinate* CalcSmoothVel(Int_t Nsmooth = 64, int densityset = 1) {
    std::vector<double> rho = densities(densityset), v(3 * (size_t)numparts_);
    nbkdt::check(nbk_smooth_vel(tree_, Nsmooth, rho_or_null(rho), v.data()));
    Coordinate* out = new Coordinate[numparts_];
    for (Int_t i = 0; i < numparts_; i++) out[i] = Coordinate(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return out;
  }
  Matrix* CalcSmoothVelDisp(Coordinate* smvel, Int_t Nsmooth = 64, int densityset = 1,
                            int meanvelset = 1) {
    std::vector<double> rho = densities(densityset);
    std::vector<double> sv = mean_velocities(smvel, meanvelset, Nsmooth, rho), d(9 * (size_t)numparts_);
    nbkdt::check(nbk_smooth_vel_disp(tree_, Nsmooth, rho_or_null(rho), sv.data(), d.data()));
    return to_matrices(d, numparts_);
  }
  Coordinate* CalcSmoothVelSkew(Coordinate* smvel, Matrix* smveldisp, Int_t Nsmooth = 64,
                                int densityset = 1, int meanvelset = 1, int veldispset = 1) {
    return moment(smvel, smveldisp, Nsmooth, densityset, meanvelset, veldispset, false);
  }
  Coordinate* CalcSmoothVelKurtosis(Coordinate* smvel, Matrix* smveldisp, Int_t Nsmooth = 64,
                                    int densityset = 1, int meanvelset = 1, int veldispset = 1) {
    return moment(smvel, smveldisp, Nsmooth, densityset, meanvelset, veldispset, true);
  }
  Double_t CalcVelDensityWithPhysDensityParticle(Int_t target, Int_t Nsmooth = 64,
                                                 Int_t Nsearch = 64, int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    int32_t t = (int32_t)target;
    double out = 0;
    nbkdt::check(nbk_veldensity_physdensity_particles(tree_, &t, 1, Nsmooth, Nsearch,
                                                      rho_or_null(rho), &out));
    return out;
  }
  Coordinate CalcSmoothVelParticle(Int_t target, Int_t Nsmooth = 64, int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    int32_t t = (int32_t)target;
    double v[3];
    nbkdt::check(nbk_smooth_vel_particles(tree_, &t, 1, Nsmooth, rho_or_null(rho), v));
    return Coordinate(v[0], v[1], v[2]);
  }
  Coordinate CalcSmoothVelPosition(Double_t* x, Int_t Nsmooth = 64, int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    double v[3];
    nbkdt::check(nbk_smooth_vel_points(tree_, x, 1, Nsmooth, rho_or_null(rho), v));
    return Coordinate(v[0], v[1], v[2]);
  }
  Coordinate CalcSmoothVelPosition(Coordinate x, Int_t Nsmooth = 64, int densityset = 1) {
    return CalcSmoothVelPosition(x.GetCoord(), Nsmooth, densityset);
  }
  Matrix CalcSmoothVelDispParticle(Int_t target, Coordinate smvel, Int_t Nsmooth = 64,
                                   int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    int32_t t = (int32_t)target;
    double sv[3] = {smvel[0], smvel[1], smvel[2]}, d[9];
    nbkdt::check(nbk_smooth_vel_disp_particles(tree_, &t, 1, Nsmooth, rho_or_null(rho), sv, d));
    return Matrix(d);
  }
  Matrix CalcSmoothVelDispPosition(Double_t* x, Coordinate smvel, Int_t Nsmooth = 64,
                                   int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    double sv[3] = {smvel[0], smvel[1], smvel[2]}, d[9];
    nbkdt::check(nbk_smooth_vel_disp_points(tree_, x, 1, Nsmooth, rho_or_null(rho), sv, d));
    return Matrix(d);
  }
  Matrix CalcSmoothVelDispPosition(Coordinate x, Coordinate smvel, Int_t Nsmooth = 64,
                                   int densityset = 1) {
    return CalcSmoothVelDispPosition(x.GetCoord(), smvel, Nsmooth, densityset);
  }
  Double_t CalcSmoothLocalMeanParticle(Int_t target, Double_t* weight, Int_t Nsmooth = 64,
                                       int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    int32_t t = (int32_t)target;
    double out = 0;
    nbkdt::check(nbk_smooth_local_mean_particles(tree_, &t, 1, Nsmooth, rho_or_null(rho),
                                                 weight, &out));
    return out;
  }
  Double_t CalcSmoothLocalMeanPosition(Double_t* x, Double_t* weight, Int_t Nsmooth = 64,
                                       int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    double out = 0;
    nbkdt::check(nbk_smooth_local_mean_points(tree_, x, 1, Nsmooth, rho_or_null(rho), weight, &out));
    return out;
  }
  Double_t CalcSmoothLocalMeanPosition(Coordinate x, Double_t* weight, Int_t Nsmooth = 64,
                                       int densityset = 1) {
    return CalcSmoothLocalMeanPosition(x.GetCoord(), weight, Nsmooth, densityset);
  }
  Double_t CalcSmoothLocalDispParticle(Int_t target, Double_t* weight, Double_t mean,
                                       Int_t Nsmooth = 64, int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    int32_t t = (int32_t)target;
    double out = 0;
    nbkdt::check(nbk_smooth_local_disp_particles(tree_, &t, 1, Nsmooth, rho_or_null(rho), weight,
                                                 &mean, &out));
    return out;
  }
  Double_t CalcSmoothLocalDispPosition(Double_t* x, Double_t* weight, Double_t mean,
                                       Int_t Nsmooth = 64, int densityset = 1) {
    std::vector<double> rho = densities(densityset);
    double out = 0;
    nbkdt::check(nbk_smooth_local_disp_points(tree_, x, 1, Nsmooth, rho_or_null(rho), weight,
                                              &mean, &out));
    return out;
  }
  Double_t CalcSmoothLocalDispPosition(Coordinate x, Double_t* weight, Double_t localmean,
                                       Int_t Nsmooth = 64, int densityset = 1) {
    return CalcSmoothLocalDispPosition(x.GetCoord(), weight, localmean, Nsmooth, densityset);
  }
  // CalcSmoothLocalValue(Nsmooth, dist, weight) (KDCalcSmoothQuantities.cxx:1721-1736): the
  // kernel sum over caller-given distances (dist[0] the largest), on the host.
  Double_t CalcSmoothLocalValue(Int_t Nsmooth, Double_t* dist, Double_t* weight) {
    std::vector<double> table(kernres_);
    double norm = 0;
    nbkdt::check(nbk_get_kernel(tree_, table.data(), &norm));
    double hi = 0.5 * dist[0];
    double hnorm = 1.0 / std::pow(hi, 3.0);
    double delta = 2.0 / (double)(kernres_ - 1), value = 0;
    for (Int_t j = 0; j < Nsmooth; j++) {
      double q = dist[j] / hi;
      int i = (int)(q * 0.5 * (kernres_ - 1));
      double w = i < kernres_ - 1 ? table[i] + (table[i + 1] - table[i]) * (q - delta * i) / delta
                                  : table[kernres_ - 1];
      value += w * hnorm * weight[j];
    }
    return value;
  }

  // ---- FOF (KDTree.h:480-503). Returns new Int_t[numparts] indexed by ID.
  Int_t* FOF(Double_t fdist, Int_t& numgroup, Int_t minnum = 8, int order = 0,
             Int_t* pHead = NULL, Int_t* pNext = NULL, Int_t* pTail = NULL, Int_t* pLen = NULL,
             int ipcheckflag = 0, FOFcheckfunc check = Pnocheck, Double_t* params = NULL) {
    (void)pHead, (void)pNext, (void)pTail, (void)pLen, (void)check, (void)params;
    if (ipcheckflag)
      throw nbkdt::Error(NBK_ERR_UNSUPPORTED, "FOF: a check function cannot run on the GPU");
    std::vector<int32_t> g(numparts_);
    int32_t ng = 0;
    nbkdt::check(nbk_fof(tree_, fdist, (int32_t)minnum, order, g.data(), &ng));
    numgroup = ng;
    Int_t* out = new Int_t[numparts_];
    for (Int_t i = 0; i < numparts_; i++) out[i] = g[i];
    return out;
  }
  Int_t* FOFCriterion(FOFcompfunc p, Double_t* params, Int_t& numgroups, Int_t minnum = 8,
                      int order = 0, int ipcheckflag = 0, FOFcheckfunc check = Pnocheck,
                      Int_t* pHead = NULL, Int_t* pNext = NULL, Int_t* pTail = NULL,
                      Int_t* pLen = NULL) {
    (void)check, (void)pHead, (void)pNext, (void)pTail, (void)pLen;
    int cmp = p == &FOF3d ? NBK_FOF3D : (p == &FOFVel ? NBK_FOFVEL : (p == &FOF6d ? NBK_FOF6D : -1));
    if (cmp < 0 || ipcheckflag)
      throw nbkdt::Error(NBK_ERR_UNSUPPORTED,
                         "FOFCriterion: only FOF3d, FOFVel and FOF6d run on the GPU");
    std::vector<int32_t> g(numparts_);
    int32_t ng = 0;
    nbkdt::check(nbk_fof_criterion(tree_, cmp, params, (int32_t)minnum, order, g.data(), &ng));
    numgroups = ng;
    Int_t* out = new Int_t[numparts_];
    for (Int_t i = 0; i < numparts_; i++) out[i] = g[i];
    return out;
  }

  // FOF over the caller's neighbour lists (KDTree.h:509-515, KDFOF.cxx:380-640): nnIDs rows
  // by tree index with numNN tree indices each (as FindNearest fills them); groups come back
  // ID-indexed and numbered by decreasing size.
  Int_t* FOFNNCriterion(FOFcompfunc p, Double_t* params, Int_t numNN, Int_t** nnIDs,
                        Int_t& numgroups, Int_t minnum = 8) {
    return fof_nn(p, params, numNN, nnIDs, nullptr, nullptr, 0, nullptr, numgroups, minnum);
  }
  // As FOFNNCriterion with params[npca[k]] = distfunc(numNN, dist2[t]) for each target t:
  // the caller's function runs here on the host, once per particle, before the GPU pass.
  Int_t* FOFNNDistCriterion(FOFcompfunc p, Double_t* params, Int_t numNN, Int_t** nnIDs,
                            Double_t** dist2, Double_t distfunc(Int_t, Double_t*), Int_t npc,
                            Int_t* npca, Int_t& numgroup, Int_t minnum = 8) {
    return fof_nn(p, params, numNN, nnIDs, dist2, distfunc, npc, npca, numgroup, minnum);
  }

  // ---- ordering (KDTree.h:522-524, KDTree.cxx:1358-1362)
  void OverWriteInputOrder() {
    iresetorder_ = false;
    for (Int_t i = 0; i < numparts_; i++) bucket_[i].SetID(i);
  }
  void SetResetOrder(bool a) { iresetorder_ = a; }

  // the underlying C-ABI handle, for batched calls (nbk_knn, nbk_knn_targets, ...)
  nbk_tree* handle() { return tree_; }

 private:
  void init(Particle* p, Int_t n, Int_t b, int treetype, int kerntype, int kernres, int split,
            int aniso, int scale, Double_t* Period, Double_t** metric, bool keep_input_order,
            Double_t rdist_adapt, Double_t adaptive_fac) {
    bucket_ = p;
    numparts_ = n;
    b_ = b;
    treetype_ = treetype;
    kerntype_ = kerntype;
    kernres_ = kernres < 100 ? 100 : kernres;  // KDTree.cxx:1145-1148
    if (metric || keep_input_order || rdist_adapt > 0 || adaptive_fac > 0)
      throw nbkdt::Error(NBK_ERR_UNSUPPORTED,
                         "KDTree: metric, keep-input-order and adaptive trees are not supported");
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), mass(n);
    for (Int_t i = 0; i < n; i++) {
      for (int j = 0; j < 3; j++) {
        pos[3 * (size_t)i + j] = p[i].GetPosition(j);
        vel[3 * (size_t)i + j] = p[i].GetVelocity(j);
      }
      mass[i] = p[i].GetMass();
    }
    if (Period)
      for (int j = 0; j < 3; j++) period_[j] = Period[j];
    nbkdt::check(nbk_create(pos.data(), vel.data(), mass.data(), n, b, treetype, kerntype,
                            kernres, split, aniso, scale, Period, 0, &tree_));
    int32_t bs;
    int64_t np_;
    nbkdt::check(nbk_get_counts(tree_, &np_, &numnodes_, &numleaves_, &bs));
    nbkdt::check(nbk_get_kernel(tree_, NULL, &kernnorm_));
    // the caller's array takes the tree's order; IDs carry the input order
    std::vector<int32_t> perm(n);
    nbkdt::check(nbk_get_perm(tree_, perm.data()));
    std::vector<Particle> old(p, p + n);
    for (Int_t t = 0; t < n; t++) {
      p[t] = old[perm[t]];
      p[t].SetID(perm[t]);
    }
  }
  void knn_one(Int_t tt, Int_t* nn, Double_t* dist2, Int_t k, int variant) {
    int32_t t = (int32_t)tt;
    std::vector<int32_t> n32(k);
    nbkdt::check(nbk_knn_targets(tree_, &t, 1, k, variant, NBK_PERIODIC_REF, n32.data(), dist2));
    for (Int_t j = 0; j < k; j++) nn[j] = n32[j];
  }
  void knn_all(Int_t** nn, Double_t** dist2, Int_t k, int variant) {
    std::vector<int32_t> n32((size_t)numparts_ * k);
    std::vector<double> d((size_t)numparts_ * k);
    nbkdt::check(nbk_knn(tree_, k, variant, NBK_PERIODIC_REF, n32.data(), d.data()));
    for (Int_t i = 0; i < numparts_; i++)
      for (Int_t j = 0; j < k; j++) {
        nn[i][j] = n32[(size_t)i * k + j];
        dist2[i][j] = d[(size_t)i * k + j];
      }
  }
  std::vector<Int_t> ball(const int32_t* target, const Double_t* x, Double_t fdist2) {
    int64_t off[2] = {0, 0}, total = 0;
    int st = target ? nbk_ball_tagged(tree_, target, 1, fdist2, off, NULL, 0, &total)
                    : nbk_ball_tagged_points(tree_, x, 1, fdist2, off, NULL, 0, &total);
    if (st != NBK_OK && st != NBK_ERR_INVALID) nbkdt::check(st);
    std::vector<int32_t> out(std::max<int64_t>(total, 1));
    nbkdt::check(target ? nbk_ball_tagged(tree_, target, 1, fdist2, off, out.data(), total, &total)
                        : nbk_ball_tagged_points(tree_, x, 1, fdist2, off, out.data(), total, &total));
    return std::vector<Int_t>(out.begin(), out.begin() + total);
  }

  Int_t* fof_nn(FOFcompfunc p, Double_t* params, Int_t numNN, Int_t** nnIDs, Double_t** dist2,
                Double_t (*distfunc)(Int_t, Double_t*), Int_t npc, Int_t* npca, Int_t& numgroups,
                Int_t minnum) {
    int cmp = p == &FOF3d ? NBK_FOF3D : (p == &FOFVel ? NBK_FOFVEL : (p == &FOF6d ? NBK_FOF6D : -1));
    if (cmp < 0)
      throw nbkdt::Error(NBK_ERR_UNSUPPORTED,
                         "FOFNNCriterion: only FOF3d, FOFVel and FOF6d run on the GPU");
    std::vector<int32_t> nn((size_t)numparts_ * numNN), g(numparts_), pidx;
    for (Int_t t = 0; t < numparts_; t++)
      for (Int_t j = 0; j < numNN; j++) nn[(size_t)t * numNN + j] = (int32_t)nnIDs[t][j];
    std::vector<double> values;
    if (distfunc) {
      values.resize(numparts_);
      for (Int_t t = 0; t < numparts_; t++) values[t] = distfunc(numNN, dist2[t]);
      for (Int_t k = 0; k < npc; k++) pidx.push_back((int32_t)npca[k]);
    }
    int32_t ng = 0;
    if (distfunc)
      nbkdt::check(nbk_fof_nn_dist_criterion(tree_, cmp, params, (int)numNN, nn.data(),
                                             values.data(), (int)npc, pidx.data(),
                                             (int32_t)minnum, g.data(), &ng));
    else
      nbkdt::check(nbk_fof_nn_criterion(tree_, cmp, params, (int)numNN, nn.data(),
                                        (int32_t)minnum, g.data(), &ng));
    numgroups = ng;
    Int_t* out = new Int_t[numparts_];
    for (Int_t i = 0; i < numparts_; i++) out[i] = g[i];
    return out;
  }

  // densities for the smoothing calls: the particles' own (densityset == 1), in ID order,
  // or none (the call computes CalcDensity(Nsmooth) first)
  std::vector<double> densities(int densityset) const {
    std::vector<double> rho;
    if (densityset == 1) {
      rho.resize(numparts_);
      for (Int_t i = 0; i < numparts_; i++) rho[bucket_[i].GetID()] = bucket_[i].GetDensity();
    }
    return rho;
  }
  static const double* rho_or_null(const std::vector<double>& rho) {
    return rho.empty() ? nullptr : rho.data();
  }
  std::vector<double> mean_velocities(const Coordinate* smvel, int meanvelset, Int_t Nsmooth,
                                      const std::vector<double>& rho) {
    std::vector<double> sv(3 * (size_t)numparts_);
    if (meanvelset == 1 && smvel) {
      for (Int_t i = 0; i < numparts_; i++)
        for (int k = 0; k < 3; k++) sv[3 * (size_t)i + k] = smvel[i][k];
    } else {
      nbkdt::check(nbk_smooth_vel(tree_, Nsmooth, rho_or_null(rho), sv.data()));
    }
    return sv;
  }
  static Matrix* to_matrices(const std::vector<double>& d, Int_t n) {
    Matrix* out = new Matrix[n];
    for (Int_t i = 0; i < n; i++)
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) out[i](k, l) = d[9 * (size_t)i + 3 * k + l];
    return out;
  }
  Coordinate* moment(const Coordinate* smvel, const Matrix* smveldisp, Int_t Nsmooth,
                     int densityset, int meanvelset, int veldispset, bool kurtosis) {
    std::vector<double> rho = densities(densityset);
    std::vector<double> sv = mean_velocities(smvel, meanvelset, Nsmooth, rho);
    std::vector<double> d(9 * (size_t)numparts_), v(3 * (size_t)numparts_);
    if (veldispset == 1 && smveldisp) {
      for (Int_t i = 0; i < numparts_; i++)
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) d[9 * (size_t)i + 3 * k + l] = smveldisp[i](k, l);
    } else {
      nbkdt::check(nbk_smooth_vel_disp(tree_, Nsmooth, rho_or_null(rho), sv.data(), d.data()));
    }
    nbkdt::check((kurtosis ? nbk_smooth_vel_kurtosis : nbk_smooth_vel_skew)(
        tree_, Nsmooth, rho_or_null(rho), sv.data(), d.data(), v.data()));
    Coordinate* out = new Coordinate[numparts_];
    for (Int_t i = 0; i < numparts_; i++) out[i] = Coordinate(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return out;
  }

  nbk_tree* tree_ = nullptr;
  Particle* bucket_ = nullptr;
  Int_t numparts_ = 0, b_ = 16;
  int treetype_ = 0, kerntype_ = 0, kernres_ = 1000;
  int64_t numnodes_ = 0, numleaves_ = 0;
  Double_t kernnorm_ = 0;
  Double_t period_[3] = {0, 0, 0};
  bool iresetorder_ = true;
};

}  // namespace NBody

#endif  // NBKDT_KDTREE_H
