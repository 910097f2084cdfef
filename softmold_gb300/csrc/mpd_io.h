// .mpd / .xyz file formats of the SoftMold `MD <name>` executable.
//
// The .mpd format is a whitespace-separated token stream of keywords, each
// followed by a fixed number of values.  Reading follows the keyword state
// machine of Blob<T>::input (include/system.h:589-1314) and its
// errorChecking() pass (include/system.h:438-580); writing reproduces the
// token sequence of Blob<T>::output (include/system.h:1315-1749) joined the
// way Script<T,U>::write does it (include/fileFormats/scriptFormat.h:64-76),
// so a file written here is byte-identical to one the reference writes for
// the same state.  The .xyz frame writer follows xyzFormat<T>::store
// (include/fileFormats/xyzFormat.h:111-143).
#pragma once

#include <array>
#include <cstdio>
#include <string>
#include <vector>

namespace smd {

// Keyword ids, in the order the reference writes them (include/system.h:292-305).
enum MpdCommand {
  CMD_GAMMA, CMD_INITIALTEMP, CMD_FINALTEMP, CMD_SEED, CMD_NTYPES, CMD_NMOLECULES,
  CMD_NPARTICLES, CMD_PERIODIC, CMD_CUTOFF, CMD_SIZE, CMD_INITIALTIME, CMD_FINALTIME,
  CMD_DELTAT, CMD_STOREINTERVAL, CMD_MEASUREINTERVAL, CMD_TWOBODYFCONST,
  CMD_TWOBODYUCONST, CMD_POSITIONS, CMD_VELOCITIES, CMD_MOLECULE, CMD_BANANA,
  CMD_DELTALXY, CMD_REMOVESOLVENT, CMD_TEMPSTEPINTERVAL, CMD_SOLVENTGAMMA,
  CMD_GAMMATYPE, CMD_TENSION, CMD_COUNT
};

// Molecule residue type ids (include/algorithms/molecules.h:6-34).
enum MoleculeType {
  MOL_CHAINOLD = 0, MOL_BENDOLD = 1, MOL_ALLPAIRS = 2, MOL_TORSION = 3, MOL_BONDOLD = 4,
  MOL_DIHEDRAL = 5, MOL_BOND = 6, MOL_BEND = 7, MOL_CHAIN = 8, MOL_BEAD = 9,
  MOL_SOLID = 10, MOL_BOUNDARY = 11, MOL_RIGIDBEND = 12, MOL_PULLBEAD = 13,
  MOL_OFFSET_BOUNDARY = 14, MOL_FLOATING_BASE = 15, MOL_ZTORQUE = 16,
  MOL_ZPOWERPOTENTIAL = 17, MOL_NANOCORE = 18, MOL_BALL = 19
};

// Constant-block sizes (include/MD.h:36-65).
constexpr int kTwoBodyConst = 6;   // nTWOBODYFCONST / nTWOBODYUCONST
constexpr int kBeadConst = 22;     // nBEADCONST
constexpr int kBeadRadius = 4;     // BEADRADIUS
constexpr int kChainConst = 4;     // nCHAINCONST: bond l0, bond k, bend a, bend k

struct Molecule {
  int type = 0;
  int nBondAlloc = 0;                       // the count read after the type
  std::vector<double> constants;
  std::vector<std::array<int, 4>> bonds;    // fourVector<int>; CHAIN: {start, nChains, length, -}
};

struct MpdSystem {
  double gamma = 0, initialTemp = 0, finalTemp = 0;
  int seed = 0, nTypes = 0, nMolecules = 0, nParticles = 0;
  bool periodic[3] = {true, true, true};
  double cutoff = 0;
  double size[3] = {0, 0, 0};
  double initialTime = 0, finalTime = 0, deltaT = 0, storeInterval = 0, measureInterval = 0;
  std::vector<double> twoBodyFconst, twoBodyUconst;
  std::vector<int> type;         // per bead
  std::vector<double> pos;       // per bead x,y,z (AoS, 3 doubles)
  std::vector<double> vel;       // per bead vx,vy,vz
  std::vector<Molecule> mol;
  double deltaLXY = 0, removeSolvent = 0, tempStepInterval = 0;
  double solventGamma[2] = {0, 0};
  std::vector<double> gammaType;
  double tension = 0;
  bool present[CMD_COUNT] = {};
};

// Number of particle indices per bond entry and number of constants for a
// molecule of the given type (include/system.h:976-1068).  Returns false for
// types written in the 4-int "default" layout.
bool molecule_layout(int type, int nTypes, int nBondAlloc, int* nIndices, int* nConstants);

// Reads <path>; returns 0 on success, else a nonzero code with a message in err.
int mpd_read_file(const std::string& path, MpdSystem& s, std::string& err);
// Parses an in-memory token stream (same rules as mpd_read_file).
int mpd_parse(const std::string& text, MpdSystem& s, std::string& err);
// Serialises exactly as Script<T,Blob>::write would.
std::string mpd_serialize(const MpdSystem& s);
int mpd_write_file(const std::string& path, const MpdSystem& s, std::string& err);

// Appends one frame to an .xyz file (xyzFormat<T>::store).
int xyz_append_frame(const std::string& path, int n, const int* type, const double* pos,
                     std::string& err);

// Formats a double the way `std::ostream << value` does with the stream's
// default precision (6), used by the .dat and .xyz writers.
std::string fmt_default(double v);

}  // namespace smd
