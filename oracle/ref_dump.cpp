// ORACLE — test infrastructure only.
//
// Golden-vector dumper compiled against the reference's own headers (by
// oracle/build_ref.sh, into oracle/_ref/).  It loads <name>.mpd with the
// reference's Script/Blob reader and writes, as raw little-endian arrays into
// <outdir>/:
//   keys.i32         CellOpt cell key of every bead (hashIndices[i].key)
//   pairs.i32        (i,j) pairs visited by CellOpt::computeForce with r<rc
//   pair_force.f64   N*3 accelerations from CellOpt::computeForce alone
//   force.f64        N*3 from computeForce + every residue's do*Force
//   energy.f64       [pair U, bonded U (CHAIN, BOND, BEND and the external-field
//                     residues), bead U (BEAD and NANOCORE), then for each scale s_k:
//                     pair dU(s_k), bonded dU(s_k), bead dU(s_k)]
//   rand53.f64       first 4096 MTRand(seed).rand53() draws
// Run with OMP_NUM_THREADS=1 so traversal and summation orders are serial.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "include/MD.h"
#include "include/system.h"

// The cell keys live in CellOpt's private hashIndices; an explicit template
// instantiation may name a private member, which lets us take its pointer.
typedef CellOpt<double, Potential<double>, Force<double> > RefCells;
struct HashIndicesTag {
  typedef keyVal<int, int>* RefCells::*type;
  friend type member_ptr(HashIndicesTag);
};
template <typename Tag, typename Tag::type M>
struct ExposeMember {
  friend typename Tag::type member_ptr(Tag) { return M; }
};
template struct ExposeMember<HashIndicesTag, &RefCells::hashIndices>;

static std::vector<std::array<int, 2>> g_pairs;

// FORCE functor that records the visited pair; positions carry the bead index
// in their type field for this pass.
template <typename T>
void RecordPair(T cutoffSquared, int nT, position<T>& p1, position<T>& p2, threeVector<T>& a1,
                threeVector<T>& a2, T* fC) {
  T dx = p1.x - p2.x;
  T dy = p1.y - p2.y;
  T dz = p1.z - p2.z;
  T dr = dx * dx + dy * dy + dz * dz;
  if (dr < cutoffSquared) g_pairs.push_back({p1.type, p2.type});
}

template <typename T>
T NoPotential(T, int, position<T>&, position<T>&, T*) {
  return 0;
}

static void write_raw(const std::string& path, const void* data, size_t bytes) {
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::cerr << "cannot write " << path << "\n";
    std::exit(2);
  }
  std::fwrite(data, 1, bytes, f);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: " << argv[0] << " name outdir [sx sy sz]...\n";
    return 1;
  }
  const std::string out = argv[2];
  Blob<double> System;
  Script<double, Blob<double> > fileIO(argv[1], std::ios::in, &System);
  fileIO.read();
  fileIO.close();
  const int N = System.readNParticles();
  position<double>* p = System.getPositions();
  threeVector<double>* acc = System.getAccelerations();

  RefCells cells(
      p, acc, System.getTwoBodyFconst(), System.getTwoBodyUconst(), N, System.readNTypes(),
      System.readSize(), System.readPeriodic(), System.readCutoff());
  cells.build();
  std::vector<int> keys(N);
  keyVal<int, int>* hashIndices = cells.*member_ptr(HashIndicesTag());
  for (int i = 0; i < N; ++i) keys[i] = hashIndices[i].key;
  write_raw(out + "/keys.i32", keys.data(), sizeof(int) * N);

  // pairs: same traversal on a copy whose type field holds the bead index
  std::vector<position<double> > pi(p, p + N);
  for (int i = 0; i < N; ++i) pi[i].type = i;
  std::vector<threeVector<double> > scratch(N);
  CellOpt<double, NoPotential<double>, RecordPair<double> > rec(
      pi.data(), scratch.data(), System.getTwoBodyFconst(), System.getTwoBodyUconst(), N,
      System.readNTypes(), System.readSize(), System.readPeriodic(), System.readCutoff());
  rec.build();
  rec.computeForce();
  write_raw(out + "/pairs.i32", g_pairs.data(), sizeof(int) * 2 * g_pairs.size());

  for (int i = 0; i < N; ++i) acc[i] = 0;
  cells.computeForce();
  std::vector<double> f(3 * (size_t)N);
  for (int i = 0; i < N; ++i) {
    f[3 * i] = acc[i].x;
    f[3 * i + 1] = acc[i].y;
    f[3 * i + 2] = acc[i].z;
  }
  write_raw(out + "/pair_force.f64", f.data(), sizeof(double) * f.size());
  for (int k = 0; k < System.readNMolecules(); ++k) {
    switch (System.getMolecule()[k].readType()) {
      case CHAIN: System.doChainForce(k); break;
      case BOND: System.doBondForce(k); break;
      case BEND: System.doBendForce(k); break;
      case BEAD: System.doBeadForce(k); break;
      case BOUNDARY: System.doBoundaryForce(k); break;
      case FLOATING_BASE: System.doFloatingBaseForce(k); break;
      case ZTORQUE: System.doZTorqueForce(k); break;
      case ZPOWERPOTENTIAL: System.doZPowerForce(k); break;
      case BALL: System.doBallForce(k); break;
      case NANOCORE: System.doNanoCoreForce(k); break;
      default: break;
    }
  }
  for (int i = 0; i < N; ++i) {
    f[3 * i] = acc[i].x;
    f[3 * i + 1] = acc[i].y;
    f[3 * i + 2] = acc[i].z;
  }
  write_raw(out + "/force.f64", f.data(), sizeof(double) * f.size());

  std::vector<double> e;
  double bonded = 0, bead = 0;
  for (int k = 0; k < System.readNMolecules(); ++k) {
    switch (System.getMolecule()[k].readType()) {
      case CHAIN: bonded += System.doChainPotential(k); break;
      case BOND: bonded += System.doBondPotential(k); break;
      case BEND: bonded += System.doBendPotential(k); break;
      case BEAD: bead += System.doBeadPotential(k); break;
      // external-field residues count with the bonded terms (the reference's
      // potential_ output sums every residue); they have no size-change term
      case BOUNDARY: bonded += System.doBoundaryPotential(k); break;
      case FLOATING_BASE: bonded += System.doFloatingBasePotential(k); break;
      case ZTORQUE: bonded += System.doZTorquePotential(k); break;
      case ZPOWERPOTENTIAL: bonded += System.doZPowerPotential(k); break;
      case BALL: bonded += System.doBallPotential(k); break;
      case NANOCORE: bead += System.doNanoCorePotential(k); break;
      default: break;
    }
  }
  e.push_back(cells.computePotential());
  e.push_back(bonded);
  e.push_back(bead);
  for (int a = 3; a + 2 < argc; a += 3) {
    threeVector<double> s;
    s.x = std::atof(argv[a]);
    s.y = std::atof(argv[a + 1]);
    s.z = std::atof(argv[a + 2]);
    double db = 0, dbead = 0;
    for (int k = 0; k < System.readNMolecules(); ++k) {
      switch (System.getMolecule()[k].readType()) {
        case CHAIN: db += System.doChainDPotential(k, s); break;
        case BOND: db += System.doBondDPotential(k, s); break;
        case BEND: db += System.doBendDPotential(k, s); break;
        case BEAD: dbead += System.doBeadDPotential(k, s); break;
        default: break;
      }
    }
    e.push_back(cells.computeDPotential(s));
    e.push_back(db);
    e.push_back(dbead);
  }
  write_raw(out + "/energy.f64", e.data(), sizeof(double) * e.size());

  MTRand r(System.readSeed());
  std::vector<double> u(4096);
  for (auto& x : u) x = r.rand53();
  write_raw(out + "/rand53.f64", u.data(), sizeof(double) * u.size());
  std::cout << N << " beads, " << g_pairs.size() << " pairs\n";
  return 0;
}
