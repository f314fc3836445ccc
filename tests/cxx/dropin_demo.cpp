// Exercises the drop-in NBody::KDTree (include/nbkdt/KDTree.h) the way reference code
// calls it (src/tests/test_kdtree.cxx, src/Analysis/Density.cxx:157-163), on particles
// read from a binary file, and writes every result keyed by particle ID so a test can
// compare it with the oracle.
//
//   dropin_demo <in.bin> <out.bin>
//   in.bin : int32 n, int32 periodic, double box, double ll, then n x (x y z vx vy vz m)
//   out.bin: int32 n, int32 numnodes, int32 numleaves, int32 ngroup,
//            n x int32 group (by ID), n x double rho (by ID, CalcDensity(32)),
//            n x 16 int32 FindNearest IDs (row by ID), n x 16 double d2,
//            int32 ball count, ball IDs, double rho after the destructor (input order),
//            n x 3 double CalcSmoothVel(32) with the stored densities (by ID),
//            int32 ngroup_nn, n x int32 FOFNNCriterion(FOF3d, 16 lists) groups (by ID),
//            n x double density after DensitySmooth(S, 16, 32) (input order),
//            phase-space tree (Aniso 0): n x 16 int32 FindNearest IDs, n x 16 double d2,
//            n x double CalcDensity(16), int32 ngroup, n x int32 FOFCriterion(FOF6d),
//            100 x double CalcDensityPosition(x + 0.01, 32) and 100 x double
//            CalcVelDensityPosition(x + 0.01, v, 16, 32) of IDs 0..99
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <nbkdt/KDTree.h>

using namespace NBody;

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  int n = 0, periodic = 0;
  double box = 0, ll = 0;
  if (fread(&n, 4, 1, f) != 1 || fread(&periodic, 4, 1, f) != 1 || fread(&box, 8, 1, f) != 1 ||
      fread(&ll, 8, 1, f) != 1)
    return 2;
  std::vector<Particle> parts(n);
  for (int i = 0; i < n; i++) {
    double v[7];
    if (fread(v, 8, 7, f) != 7) return 2;
    for (int j = 0; j < 3; j++) {
      parts[i].SetPosition(j, v[j]);
      parts[i].SetVelocity(j, v[3 + j]);
    }
    parts[i].SetMass(v[6]);
    parts[i].SetPID(i);
  }
  fclose(f);
  double period[3] = {box, box, box};
  std::vector<int> group(n), nnid((size_t)n * 16), ballid, group_nn(n);
  int ngroup_nn = 0;
  std::vector<double> rho(n), d2((size_t)n * 16), rho_after(n), smvel(3 * (size_t)n);
  std::vector<double> posden(100), posvden(100);
  int numnodes, numleaves, ngroup = 0;
  {
    KDTree tree(parts.data(), n, 16, KDTree::TPHYS, KDTree::KSPH, 1000, 0, 0, 0,
                periodic ? period : NULL);
    numnodes = tree.GetNumNodes();
    numleaves = tree.GetNumLeafNodes();
    // IDs follow the particles (KDTree.cxx:1291)
    Int_t* g = tree.FOF(ll, ngroup, 20);
    for (int i = 0; i < n; i++) group[i] = g[i];
    delete[] g;
    tree.CalcDensity(32);
    for (int t = 0; t < n; t++) rho[parts[t].GetID()] = parts[t].GetDensity();
    // densityset = 1: the densities CalcDensity stored in the particles
    Coordinate* sv = tree.CalcSmoothVel(32, 1);
    for (int i = 0; i < n; i++)
      for (int k = 0; k < 3; k++) smvel[3 * (size_t)i + k] = sv[i][k];
    delete[] sv;
    std::vector<Int_t> nn(16);
    std::vector<Double_t> dd(16);
    std::vector<Int_t> flat((size_t)n * 16);
    std::vector<Int_t*> rows(n);
    for (int t = 0; t < n; t++) {
      tree.FindNearest(t, nn.data(), dd.data(), 16);
      int id = parts[t].GetID();
      rows[t] = &flat[(size_t)t * 16];
      for (int j = 0; j < 16; j++) {
        nnid[(size_t)id * 16 + j] = parts[nn[j]].GetID();
        d2[(size_t)id * 16 + j] = dd[j];
        rows[t][j] = nn[j];  // tree indices, as the reference's lists
      }
    }
    Double_t fof_params[8] = {0, 0, 0, 0, 0, 0, 0.35, 0};
    Int_t ngn = 0;
    Int_t* gn = tree.FOFNNCriterion(FOF3d, fof_params, 16, rows.data(), ngn, 5);
    for (int i = 0; i < n; i++) group_nn[i] = gn[i];
    ngroup_nn = ngn;
    delete[] gn;
    // the tree index of ID 0
    int t0 = 0;
    while (parts[t0].GetID() != 0) t0++;
    std::vector<Int_t> tagged = tree.SearchBallPosTagged(t0, 4 * ll * ll);
    for (Int_t t : tagged) ballid.push_back(parts[t].GetID());
    // CalcDensityPosition / CalcVelDensityPosition next to the first 100 particles (by ID)
    for (int t = 0; t < n; t++) {
      int id = parts[t].GetID();
      if (id >= 100) continue;
      Double_t x[3], vq[3];
      for (int k = 0; k < 3; k++) {
        x[k] = parts[t].GetPosition(k) + 0.01;
        vq[k] = parts[t].GetVelocity(k);
      }
      posden[id] = tree.CalcDensityPosition(x, 32);
      posvden[id] = tree.CalcVelDensityPosition(x, vq, 16, 32);
    }
  }
  // the destructor restored input order
  for (int i = 0; i < n; i++) rho_after[i] = parts[i].GetDensity();
  // DensitySmooth(System&, b, k) of src/Analysis/Density.cxx:157-163, the reference's
  // in-repo caller: a System-constructed tree (default kernel) and CalcDensity
  std::vector<double> rho_smooth(n);
  {
    System S(n, parts.data());
    KDTree* tree = new KDTree(S, 16);
    tree->CalcDensity(32);
    delete tree;
    for (int i = 0; i < n; i++) rho_smooth[i] = S[i].GetDensity();
  }
  // a phase-space tree (TreeType TPHS, Aniso 0, the reference's default): FindNearest for
  // every particle (the Int_t** form, rows by tree index), CalcDensity and
  // FOFCriterion(FOF6d); the destructor restores input order again
  std::vector<int> pnn((size_t)n * 16), pgroup(n);
  std::vector<double> pd2((size_t)n * 16), prho(n);
  int pngroup = 0;
  {
    KDTree ptree(parts.data(), n, 16, KDTree::TPHS, KDTree::KSPH, 1000, 0, 0, 0,
                 periodic ? period : NULL);
    std::vector<Int_t> flat((size_t)n * 16);
    std::vector<Double_t> dflat((size_t)n * 16);
    std::vector<Int_t*> r(n);
    std::vector<Double_t*> dr(n);
    for (int t = 0; t < n; t++) {
      r[t] = &flat[(size_t)t * 16];
      dr[t] = &dflat[(size_t)t * 16];
    }
    ptree.FindNearest(r.data(), dr.data(), 16);
    for (int t = 0; t < n; t++) {
      int id = parts[t].GetID();
      for (int j = 0; j < 16; j++) {
        pnn[(size_t)id * 16 + j] = parts[r[t][j]].GetID();
        pd2[(size_t)id * 16 + j] = dr[t][j];
      }
    }
    ptree.CalcDensity(16);
    for (int t = 0; t < n; t++) prho[parts[t].GetID()] = parts[t].GetDensity();
    Double_t par[20] = {(Double_t)KDTree::TPHS, 0.25, 0.04, 0, 0, 0, 0.25, 0.04};
    Int_t* g6 = ptree.FOFCriterion(FOF6d, par, pngroup, 8);
    for (int i = 0; i < n; i++) pgroup[i] = g6[i];
    delete[] g6;
  }
  FILE* o = fopen(argv[2], "wb");
  fwrite(&n, 4, 1, o);
  fwrite(&numnodes, 4, 1, o);
  fwrite(&numleaves, 4, 1, o);
  fwrite(&ngroup, 4, 1, o);
  fwrite(group.data(), 4, n, o);
  fwrite(rho.data(), 8, n, o);
  fwrite(nnid.data(), 4, (size_t)n * 16, o);
  fwrite(d2.data(), 8, (size_t)n * 16, o);
  int nb = (int)ballid.size();
  fwrite(&nb, 4, 1, o);
  fwrite(ballid.data(), 4, nb, o);
  fwrite(rho_after.data(), 8, n, o);
  fwrite(smvel.data(), 8, 3 * (size_t)n, o);
  fwrite(&ngroup_nn, 4, 1, o);
  fwrite(group_nn.data(), 4, n, o);
  fwrite(rho_smooth.data(), 8, n, o);
  fwrite(pnn.data(), 4, (size_t)n * 16, o);
  fwrite(pd2.data(), 8, (size_t)n * 16, o);
  fwrite(prho.data(), 8, n, o);
  fwrite(&pngroup, 4, 1, o);
  fwrite(pgroup.data(), 4, n, o);
  fwrite(posden.data(), 8, 100, o);
  fwrite(posvden.data(), 8, 100, o);
  fclose(o);
  printf("dropin ok: n=%d nodes=%d groups=%d\n", n, numnodes, ngroup);
  return 0;
}
