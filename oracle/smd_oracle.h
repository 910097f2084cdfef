// ORACLE — test infrastructure only.
//
// CPU restatement of the SoftMold implicit-solvent MD step (the reference's
// MD.cpp loop and the CellOpt / Blob / Verlet / Langevin code it calls).  It
// checks the CUDA library's results: only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline arm may load or run it, never the product path.
//
// Parity of this restatement is pinned by golden vectors dumped from the
// reference's own code (oracle/ref_dump.cpp compiled against the reference
// headers by oracle/build_ref.sh) and committed under tests/golden/.
//
// Arrays are plain C: positions/velocities/forces are N*3 doubles (AoS x,y,z),
// types are N ints, constant tables are the reference's flat layouts.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// OpenMP threads used by the pair and chain passes (1 = the reference's
// serial order, which makes results bit-identical).
void orc_set_threads(int n);

// MT19937 (Matsumoto & Nishimura 1998) with the 53-bit real draw used by the
// reference's MTRand::rand53 (include/algorithms/MersenneTwister.h:337-341).
typedef struct {
  uint32_t state[624];
  int left;
  int next;
} orc_mt;
void orc_mt_seed(orc_mt* g, uint32_t seed);
uint32_t orc_mt_u32(orc_mt* g);
double orc_mt_rand53(orc_mt* g);
void orc_mt_fill53(uint32_t seed, int n, double* out);

// Cell key of each bead (include/algorithms/cellOpt.h:532-555).
void orc_cell_keys(int n, const double* pos, const double box[3], double rc, int* keys);

// Pairs visited by CellOpt::computeForce with r^2 < rc^2, in visiting order
// (include/algorithms/cellOpt.h:712-926).  Returns the pair count (writes at
// most cap pairs as (i,j)), or -1 if a cell holds more than 512 beads.
long orc_pair_list(int n, const double* pos, const double box[3], double rc, int* pairs, long cap);

// a += non-bonded forces (CellOpt::computeForce with Force, include/MD.h:795-848).
int orc_pair_force(int n, const double* pos, const int* type, const double box[3], double rc,
                   int nTypes, const double* fconst, double* acc);
// Sum of non-bonded potentials (CellOpt::computePotential, include/MD.h:895-930).
double orc_pair_potential(int n, const double* pos, const int* type, const double box[3], double rc,
                          int nTypes, const double* uconst);
// Sum over the current cell list's pairs of U(d) - U(s*d) (CellOpt::computeDPotential).
double orc_pair_dpotential(int n, const double* pos, const int* type, const double box[3], double rc,
                           int nTypes, const double* uconst, const double scale[3]);

// CHAIN residue (start, nChains, length) with constants {l0, kbond, abend, kbend}:
// forces (Blob::doChainForce, include/system.h:1782-1866), potential
// (doChainPotential, :2487-2568) and size-change difference (doChainDPotential, :3280-3384).
void orc_chain_force(const double* pos, const double box[3], int start, int nChains, int length,
                     const double* c, double* acc);
double orc_chain_potential(const double* pos, const double box[3], int start, int nChains, int length,
                           const double* c);
double orc_chain_dpotential(const double* pos, const double box[3], int start, int nChains,
                            int length, const double* c, const double scale[3]);

// BOND residue: nb pairs list[2k], list[2k+1], constants {l0, k}: forces
// (Blob::doBondForce, include/system.h:1880-1934), potential (doBondPotential,
// :2718-2745), size-change difference (doBondDPotential, :3399-3435).
void orc_bond_force(const double* pos, const double box[3], int nb, const int* list, const double* c, double* acc);
double orc_bond_potential(const double* pos, const double box[3], int nb, const int* list, const double* c);
double orc_bond_dpotential(const double* pos, const double box[3], int nb, const int* list, const double* c,
                           const double scale[3]);

// BEND residue: nb triplets list[3k..3k+2], constants {a, k}: forces
// (Blob::doBendForce, include/system.h:1975-2040), potential (doBendPotential,
// :2782-2821), size-change difference (doBendDPotential, :3477-3524).
void orc_bend_force(const double* pos, const double box[3], int nb, const int* list, const double* c, double* acc);
double orc_bend_potential(const double* pos, const double box[3], int nb, const int* list, const double* c);
double orc_bend_dpotential(const double* pos, const double box[3], int nb, const int* list, const double* c,
                           const double scale[3]);

// BEAD residue (continuum spheres) with bead indices idx[nb], constants
// C[22*nTypes*nTypes]: force (Blob::doBeadForce brute-force branch,
// include/system.h:2043-2212), potential (doBeadPotential, :2936-3074) and
// size-change difference (doBeadDPotential, :3584-3700).
void orc_bead_force(int n, const double* pos, const int* type, const double box[3], int nTypes,
                    int nb, const int* idx, const double* C, double* acc);
double orc_bead_potential(int n, const double* pos, const int* type, const double box[3], int nTypes,
                          int nb, const int* idx, const double* C);
double orc_bead_dpotential(int n, const double* pos, const int* type, const double box[3], int nTypes,
                           int nb, const int* idx, const double* C, const double scale[3]);

// External-field residues.  Forces and potentials, no size-change
// difference: the reference's barostat adds none for them (MD.cpp:640-656).
// BOUNDARY: beads[nb], constants {dim, centre, -, k} (Blob::doBoundaryForce /
// doBoundaryPotential, include/system.h:2335-2349, 3138-3151; boundaryF /
// boundaryP, include/MD.h:546-617).
void orc_boundary_force(const double* pos, const double box[3], int nb, const int* beads, const double* c,
                        double* acc);
double orc_boundary_potential(const double* pos, const double box[3], int nb, const int* beads, const double* c);
// FLOATING_BASE: beads[nb], constants 6 per bead type (Blob::doFloatingBaseForce
// / doFloatingBasePotential, include/system.h:2403-2447; floatingBaseForce /
// floatingBasePotential, include/MD.h:458-497).
void orc_floating_base_force(const double* pos, const int* type, int nb, const int* beads, const double* c,
                             double* acc);
double orc_floating_base_potential(const double* pos, const int* type, int nb, const int* beads, const double* c);
// ZPOWERPOTENTIAL: blocks {start, count}[nb], constants {c0, c1}
// (Blob::doZPowerForce / doZPowerPotential, include/system.h:2666-2716;
// zPowerForce / zPowerPotential, include/MD.h:1143-1154).
void orc_zpower_force(const double* pos, int nb, const int* blocks, const double* c, double* acc);
double orc_zpower_potential(const double* pos, int nb, const int* blocks, const double* c);
// ZTORQUE: blocks {start, nChains, length}[nb], constants {a, b, c, z0}
// (Blob::doZTorqueForce / doZTorquePotential, include/system.h:2583-2664;
// zTorqueForce / zTorquePotential, include/MD.h:1116-1141).
void orc_ztorque_force(const double* pos, const double box[3], int nb, const int* blocks, const double* c,
                       double* acc);
double orc_ztorque_potential(const double* pos, const double box[3], int nb, const int* blocks, const double* c);

// BALL: bonds {first, second}[nb], constants {r0, k}: harmonicHalfF on each
// bond, all pulling the first bond's first bead; the potential takes each
// bond's own first bead (Blob::doBallForce / doBallPotential,
// include/system.h:1937-1971, 2750-2779; harmonicHalfF / harmonicHalfP,
// include/MD.h:1164-1222).
void orc_ball_force(const double* pos, const double box[3], int nb, const int* bonds, const double* c, double* acc);
double orc_ball_potential(const double* pos, const double box[3], int nb, const int* bonds, const double* c);

// NANOCORE: cores idx[nb], 22 constants per core C[22*nb]: each core against
// every other bead (other cores included) with its own constants, brute force
// as the reference does below 50 cores (Blob::doNanoCoreForce /
// doNanoCorePotential, include/system.h:2216-2263, 3029-3073).
void orc_nanocore_force(int n, const double* pos, const double box[3], int nb, const int* idx, const double* C,
                        double* acc);
double orc_nanocore_potential(int n, const double* pos, const double box[3], int nb, const int* idx,
                              const double* C);

// Runs the reference MD loop on <name>.mpd exactly as `MD <name>` does
// (MD.cpp:72-755) with `threads` OpenMP threads (1 reproduces the reference's
// single-thread random streams).  Returns 0 on success.
int orc_md_run(const char* name, int threads);

// Times `steps` loop iterations of the restated step on the system in
// <name>.mpd without any file output; returns elapsed seconds (<0 on error).
double orc_md_time(const char* name, int threads, int steps);

#ifdef __cplusplus
}
#endif
