// .mpd / .xyz readers and writers; see mpd_io.h for the reference interfaces.
#include "mpd_io.h"

#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>

namespace smd {

namespace {

const char* const kCommandNames[CMD_COUNT] = {
    "gamma",       "initialTemp",   "finalTemp",       "seed",          "nTypes",
    "nMolecules",  "nParticles",    "periodic",        "cutoff",        "size",
    "initialTime", "finalTime",     "deltaT",          "storeInterval", "measureInterval",
    "twoBodyFconst", "twoBodyUconst", "positions",     "velocities",    "molecule",
    "banana",      "deltaLXY",      "removeSolvent",   "tempStepInterval",
    "solventGamma", "gammaType",    "tension"};

template <typename V>
bool parse_token(const std::string& tok, V& out) {
  std::stringstream ss(tok);
  ss >> out;
  return !ss.fail();
}

std::string fmt15(double v) {
  std::ostringstream o;
  o << std::setprecision(15) << v;
  return o.str();
}
std::string fmt15(int v) {
  std::ostringstream o;
  o << v;
  return o.str();
}

// Cursor over the token stream.  Script<T,U>::read stops at the first "end"
// token and drops a final token that is not followed by whitespace
// (include/fileFormats/scriptFormat.h:79-94).
struct Tokens {
  std::vector<std::string> t;
  size_t i = 0;
  bool next(std::string& out) {
    if (i >= t.size()) return false;
    out = t[i++];
    return true;
  }
  size_t left() const { return t.size() - i; }
};

// Bounds on counts read from the file that size products below: nTypes keeps
// kBeadConst * nTypes^2 (a BEAD residue's constants) within an int, and
// nBondAlloc keeps kBeadConst * nBondAlloc (a NANOCORE residue's) within one.
constexpr int kMaxTypesRead = 4096;
constexpr int kMaxBondAllocRead = 1 << 26;

Tokens tokenize(const std::string& text) {
  Tokens tk;
  std::istringstream in(text);
  std::string s;
  while (true) {
    in >> s;
    if (in.eof()) break;  // the reference ignores a token that hits end-of-file
    if (in.fail()) break;
    if (s == "end") break;
    tk.t.push_back(s);
  }
  return tk;
}

}  // namespace

std::string fmt_default(double v) {
  std::ostringstream o;
  o << v;
  return o.str();
}

bool molecule_layout(int type, int nTypes, int nBondAlloc, int* nIdx, int* nConst) {
  switch (type) {
    case MOL_BOND: *nIdx = 2; *nConst = 2; return true;
    case MOL_BEND: *nIdx = 3; *nConst = 2; return true;
    case MOL_CHAIN: *nIdx = 3; *nConst = kChainConst; return true;
    case MOL_BEAD: *nIdx = 1; *nConst = kBeadConst * nTypes * nTypes; return true;
    case MOL_SOLID: *nIdx = 1; *nConst = 1; return true;
    case MOL_BOUNDARY: *nIdx = 1; *nConst = 4; return true;
    case MOL_OFFSET_BOUNDARY: *nIdx = 1; *nConst = 4; return true;
    case MOL_RIGIDBEND: *nIdx = 2; *nConst = 5; return true;
    case MOL_PULLBEAD: *nIdx = 1; *nConst = 4; return true;
    case MOL_FLOATING_BASE: *nIdx = 1; *nConst = 6 * nTypes; return true;
    case MOL_ZTORQUE: *nIdx = 3; *nConst = 4; return true;
    case MOL_ZPOWERPOTENTIAL: *nIdx = 2; *nConst = 2; return true;
    case MOL_NANOCORE: *nIdx = 1; *nConst = kBeadConst * nBondAlloc; return true;
    case MOL_BALL: *nIdx = 2; *nConst = 2; return true;
    default: *nIdx = 0; *nConst = 0; return false;  // TORSION, DIHEDRAL, unknown
  }
}

int mpd_parse(const std::string& text, MpdSystem& s, std::string& err) {
  std::map<std::string, int> lookup;
  for (int c = 0; c < CMD_COUNT; ++c) lookup[kCommandNames[c]] = c;
  Tokens tk = tokenize(text);
  std::string tok;
  auto need = [&](const char* what) -> bool {
    if (!tk.next(tok)) {
      err = std::string("Value after ") + what + " is missing (end of file)";
      return false;
    }
    return true;
  };
  auto read_d = [&](const char* what, double& out) -> bool {
    if (!need(what)) return false;
    if (!parse_token(tok, out)) {
      err = std::string("Value after ") + what + " is not a numerical type!";
      return false;
    }
    return true;
  };
  auto read_i = [&](const char* what, int& out) -> bool {
    if (!need(what)) return false;
    if (!parse_token(tok, out)) {
      err = std::string("Value after ") + what + " is not a numerical type!";
      return false;
    }
    return true;
  };
  // The arrays below are sized from counts in the file.  A negative count
  // fails at once, and one whose entries the rest of the file cannot hold
  // fails as the missing value would, before anything is allocated for it.
  auto room = [&](const char* what, double entries) -> bool {
    if (entries < 0) {
      err = std::string("Count for ") + what + " is negative!";
      return false;
    }
    if (entries > (double)tk.left()) {
      err = std::string("Value after ") + what + " is missing (end of file)";
      return false;
    }
    return true;
  };
  bool haveVel = false;
  while (tk.next(tok)) {
    auto f = lookup.find(tok);
    if (f == lookup.end()) {
      err = tok + " is not a recognized command!";
      return 1;
    }
    const int c = f->second;
    const char* name = kCommandNames[c];
    switch (c) {
      case CMD_GAMMA: if (!read_d(name, s.gamma)) return 2; break;
      case CMD_INITIALTEMP: if (!read_d(name, s.initialTemp)) return 2; break;
      case CMD_FINALTEMP: if (!read_d(name, s.finalTemp)) return 2; break;
      case CMD_SEED: if (!read_i(name, s.seed)) return 2; break;
      case CMD_NTYPES:
        if (!read_i(name, s.nTypes)) return 2;
        if (s.nTypes < 0 || s.nTypes > kMaxTypesRead) {
          err = "nTypes must be in 0.." + std::to_string(kMaxTypesRead) + "!";
          return 3;
        }
        break;
      case CMD_NMOLECULES: if (!read_i(name, s.nMolecules)) return 2; break;
      case CMD_NPARTICLES: if (!read_i(name, s.nParticles)) return 2; break;
      case CMD_PERIODIC:
        // The value is consumed and ignored: periodic boundaries are always on.
        if (!need(name)) return 2;
        s.periodic[0] = s.periodic[1] = s.periodic[2] = true;
        break;
      case CMD_CUTOFF: if (!read_d(name, s.cutoff)) return 2; break;
      case CMD_SIZE:
        for (int d = 0; d < 3; ++d) if (!read_d(name, s.size[d])) return 2;
        break;
      case CMD_INITIALTIME: if (!read_d(name, s.initialTime)) return 2; break;
      case CMD_FINALTIME: if (!read_d(name, s.finalTime)) return 2; break;
      case CMD_DELTAT: if (!read_d(name, s.deltaT)) return 2; break;
      case CMD_STOREINTERVAL: if (!read_d(name, s.storeInterval)) return 2; break;
      case CMD_MEASUREINTERVAL: if (!read_d(name, s.measureInterval)) return 2; break;
      case CMD_TWOBODYFCONST:
      case CMD_TWOBODYUCONST: {
        if (!s.present[CMD_NTYPES]) {
          err = std::string("nTypes was not present before ") + name + "!";
          return 3;
        }
        std::vector<double>& dst = (c == CMD_TWOBODYFCONST) ? s.twoBodyFconst : s.twoBodyUconst;
        const int n = kTwoBodyConst * s.nTypes * s.nTypes;
        if (!room(name, n)) return 2;
        dst.assign(n, 0.0);
        for (int k = 0; k < n; ++k) if (!read_d(name, dst[k])) return 2;
        break;
      }
      case CMD_POSITIONS: {
        if (!s.present[CMD_NPARTICLES]) {
          err = "nParticles was not present before positions!";
          return 3;
        }
        if (!room(name, 4.0 * s.nParticles)) return 2;
        s.type.assign(s.nParticles, 0);
        s.pos.assign(3 * (size_t)s.nParticles, 0.0);
        for (int p = 0; p < s.nParticles; ++p) {
          if (!read_i(name, s.type[p])) return 2;
          for (int d = 0; d < 3; ++d) if (!read_d(name, s.pos[3 * (size_t)p + d])) return 2;
        }
        break;
      }
      case CMD_VELOCITIES: {
        if (!s.present[CMD_NPARTICLES]) {
          err = "nParticles was not present before velocities!";
          return 3;
        }
        if (!room(name, 3.0 * s.nParticles)) return 2;
        s.vel.assign(3 * (size_t)s.nParticles, 0.0);
        for (size_t k = 0; k < 3 * (size_t)s.nParticles; ++k) if (!read_d(name, s.vel[k])) return 2;
        haveVel = true;
        break;
      }
      case CMD_MOLECULE: {
        if (!s.present[CMD_NMOLECULES]) {
          err = "nMolecules was not present before molecules!";
          return 3;
        }
        s.mol.clear();
        for (int m = 0; m < s.nMolecules; ++m) {
          Molecule mol;
          if (!read_i(name, mol.type)) return 2;
          int nIdx, nConst;
          if (!molecule_layout(mol.type, s.nTypes, 0, &nIdx, &nConst)) {
            std::array<int, 4> b{0, 0, 0, 0};
            for (int k = 0; k < 4; ++k) if (!read_i(name, b[k])) return 2;
            mol.bonds.push_back(b);
            mol.nBondAlloc = 1;
          } else {
            if (mol.type == MOL_BEAD && s.nTypes <= 0) {
              err = "nTypes undefined for BEAD molecule!";
              return 3;
            }
            if (!read_i(name, mol.nBondAlloc)) return 2;
            if (mol.nBondAlloc < 0 || mol.nBondAlloc > kMaxBondAllocRead) {
              err = "Molecule " + std::to_string(m) + ": bond count out of range!";
              return 3;
            }
            molecule_layout(mol.type, s.nTypes, mol.nBondAlloc, &nIdx, &nConst);
            if (!room(name, (double)nConst + (double)nIdx * mol.nBondAlloc)) return 2;
            mol.constants.assign(nConst, 0.0);
            for (int k = 0; k < nConst; ++k) if (!read_d(name, mol.constants[k])) return 2;
            for (int b = 0; b < mol.nBondAlloc; ++b) {
              std::array<int, 4> bond{0, 0, 0, 0};
              for (int k = 0; k < nIdx; ++k) if (!read_i(name, bond[k])) return 2;
              mol.bonds.push_back(bond);
            }
          }
          s.mol.push_back(std::move(mol));
        }
        break;
      }
      case CMD_BANANA: break;
      case CMD_DELTALXY: if (!read_d(name, s.deltaLXY)) return 2; break;
      case CMD_REMOVESOLVENT: if (!read_d(name, s.removeSolvent)) return 2; break;
      case CMD_TEMPSTEPINTERVAL: if (!read_d(name, s.tempStepInterval)) return 2; break;
      case CMD_SOLVENTGAMMA:
        for (int k = 0; k < 2; ++k) if (!read_d(name, s.solventGamma[k])) return 2;
        break;
      case CMD_GAMMATYPE:
        if (!s.present[CMD_NTYPES]) {
          err = "nTypes was not present before gammaType!";
          return 3;
        }
        if (!room(name, s.nTypes)) return 2;
        s.gammaType.assign(s.nTypes, 0.0);
        for (int k = 0; k < s.nTypes; ++k) if (!read_d(name, s.gammaType[k])) return 2;
        break;
      case CMD_TENSION: if (!read_d(name, s.tension)) return 2; break;
    }
    s.present[c] = true;
  }
  // errorChecking() (include/system.h:438-580)
  const size_t np = s.nParticles;
  if (s.type.size() != np || !haveVel || s.vel.size() != 3 * np) {
    std::ostringstream o;
    o << "Mismatch of parameters: nParticles " << s.nParticles << ", positions " << s.type.size()
      << ", velocities " << (haveVel ? s.vel.size() / 3 : 0);
    err = o.str();
    return 4;
  }
  for (size_t i = 0; i < np; ++i) {
    for (int d = 0; d < 3; ++d) {
      const double x = s.pos[3 * i + d];
      if (x > s.size[d] || x < 0) {
        std::ostringstream o;
        o << "XYZ"[d] << " position of particle " << i << " is out of bounds.";
        err = o.str();
        return 5;
      }
    }
  }
  for (size_t m = 0; m < s.mol.size(); ++m) {
    const Molecule& mol = s.mol[m];
    for (size_t b = 0; b < mol.bonds.size(); ++b) {
      const auto& bd = mol.bonds[b];
      bool bad = false;
      if (mol.type == MOL_BOND) bad = bd[0] > s.nParticles || bd[1] > s.nParticles || bd[0] < 0 || bd[1] < 0;
      if (mol.type == MOL_BEND)
        bad = bd[0] > s.nParticles || bd[1] > s.nParticles || bd[2] > s.nParticles || bd[0] < 0 ||
              bd[1] < 0 || bd[2] < 0;
      if (mol.type == MOL_CHAIN) {
        const long end = (long)bd[0] + (long)bd[1] * (long)bd[2];
        bad = end > s.nParticles || end < 0;
      }
      if (bad) {
        std::ostringstream o;
        o << "Molecule " << m << ", bond " << b << " is out of bounds!";
        err = o.str();
        return 6;
      }
    }
  }
  return 0;
}

int mpd_read_file(const std::string& path, MpdSystem& s, std::string& err) {
  std::ifstream f(path);
  if (!f.is_open()) {
    err = "Could not open " + path;
    return 10;
  }
  std::stringstream buf;
  buf << f.rdbuf();
  return mpd_parse(buf.str(), s, err);
}

std::string mpd_serialize(const MpdSystem& s) {
  std::string out;
  auto emit = [&](const std::string& tok) {
    out += tok;
    out += ' ';
  };
  for (int c = 0; c < CMD_COUNT; ++c) {
    if (!s.present[c]) {
      emit("");  // an absent keyword still produces a separator
      continue;
    }
    emit((c != 0 ? std::string("\n") : std::string()) + kCommandNames[c]);
    switch (c) {
      case CMD_GAMMA: emit(fmt15(s.gamma)); break;
      case CMD_INITIALTEMP: emit(fmt15(s.initialTemp)); break;
      case CMD_FINALTEMP: emit(fmt15(s.finalTemp)); break;
      case CMD_SEED: emit(fmt15(s.seed)); break;
      case CMD_NTYPES: emit(fmt15(s.nTypes)); break;
      case CMD_NMOLECULES: emit(fmt15(s.nMolecules)); break;
      case CMD_NPARTICLES: emit(fmt15(s.nParticles)); break;
      case CMD_PERIODIC: emit(fmt15((int)s.periodic[0])); break;
      case CMD_CUTOFF: emit(fmt15(s.cutoff)); break;
      case CMD_SIZE: for (int d = 0; d < 3; ++d) emit(fmt15(s.size[d])); break;
      case CMD_INITIALTIME: emit(fmt15(s.initialTime)); break;
      case CMD_FINALTIME: emit(fmt15(s.finalTime)); break;
      case CMD_DELTAT: emit(fmt15(s.deltaT)); break;
      case CMD_STOREINTERVAL: emit(fmt15(s.storeInterval)); break;
      case CMD_MEASUREINTERVAL: emit(fmt15(s.measureInterval)); break;
      case CMD_TWOBODYFCONST:
      case CMD_TWOBODYUCONST: {
        const std::vector<double>& v = (c == CMD_TWOBODYFCONST) ? s.twoBodyFconst : s.twoBodyUconst;
        const size_t n = (size_t)kTwoBodyConst * s.nTypes * s.nTypes;
        for (size_t it = 1; it <= n; ++it) {
          std::string t = (it == 1) ? "\n " : "";
          t += fmt15(it - 1 < v.size() ? v[it - 1] : 0.0);
          if (it % kTwoBodyConst == 0) t += "\n";
          emit(t);
        }
        break;
      }
      case CMD_POSITIONS: {
        const size_t n = 4 * (size_t)s.nParticles;
        for (size_t it = 1; it <= n; ++it) {
          const size_t p = (it - 1) / 4, k = (it - 1) % 4;
          std::string t = (it == 1) ? "\n " : "";
          t += (k == 0) ? fmt15(s.type[p]) : fmt15(s.pos[3 * p + k - 1]);
          if (k == 3) t += "\n";
          emit(t);
        }
        break;
      }
      case CMD_VELOCITIES: {
        const size_t n = 3 * (size_t)s.nParticles;
        for (size_t it = 1; it <= n; ++it) {
          std::string t = (it == 1) ? "\n " : "";
          t += fmt15(s.vel[it - 1]);
          if ((it - 1) % 3 == 2) t += "\n";
          emit(t);
        }
        break;
      }
      case CMD_MOLECULE: {
        for (size_t m = 0; m < s.mol.size(); ++m) {
          const Molecule& mol = s.mol[m];
          emit((m == 0 ? std::string("\n") : std::string()) + fmt15(mol.type) + "\t");
          int nIdx, nConst;
          if (!molecule_layout(mol.type, s.nTypes, (int)mol.bonds.size(), &nIdx, &nConst)) {
            for (int k = 0; k < 4; ++k) emit(fmt15(mol.bonds.empty() ? 0 : mol.bonds[0][k]));
            continue;
          }
          emit(fmt15((int)mol.bonds.size()) + "\n");
          for (int k = 1; k <= nConst; ++k) {
            std::string t = fmt15(k - 1 < (int)mol.constants.size() ? mol.constants[k - 1] : 0.0) + " ";
            if (k % kBeadConst == 0 && mol.type == MOL_BEAD) t += "\n";
            if (k == nConst) t += "\n";
            emit(t);
          }
          for (const auto& b : mol.bonds) {
            for (int k = 0; k < nIdx; ++k) {
              std::string t = fmt15(b[k]) + " ";
              if (k == nIdx - 1) t += "\n";
              emit(t);
            }
          }
        }
        break;
      }
      case CMD_BANANA: emit("\n"); break;
      case CMD_DELTALXY: emit(fmt15(s.deltaLXY)); break;
      case CMD_REMOVESOLVENT: emit(fmt15(s.removeSolvent)); break;
      case CMD_TEMPSTEPINTERVAL: emit(fmt15(s.tempStepInterval)); break;
      case CMD_SOLVENTGAMMA: for (int k = 0; k < 2; ++k) emit(fmt15(s.solventGamma[k])); break;
      case CMD_GAMMATYPE: for (int k = 0; k < s.nTypes; ++k) emit(fmt15(s.gammaType[k])); break;
      case CMD_TENSION: emit(fmt15(s.tension)); break;
    }
  }
  out += '\n';
  return out;
}

// The file is written beside its target and renamed over it, so a run that
// dies while storing leaves the previous checkpoint whole (MDcuda keeps a
// second copy for the same purpose, MDcuda.cu:87-112, 353-360); the bytes
// and the final file set are those of a direct write.
int mpd_write_file(const std::string& path, const MpdSystem& s, std::string& err) {
  const std::string tmp = path + ".part";
  std::ofstream f(tmp, std::ios::out | std::ios::trunc);
  if (!f.is_open()) {
    err = "Could not open " + tmp + " for writing";
    return 10;
  }
  f << mpd_serialize(s);
  f.close();
  if (f.fail()) {
    std::remove(tmp.c_str());
    err = "Write failed for " + tmp;
    return 11;
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) {
    std::remove(tmp.c_str());
    err = "Could not replace " + path;
    return 12;
  }
  return 0;
}

int xyz_append_frame(const std::string& path, int n, const int* type, const double* pos,
                     std::string& err) {
  std::ofstream f(path, std::ios::out | std::ios::app);
  if (!f.is_open()) {
    err = "Could not open " + path;
    return 10;
  }
  std::ostringstream o;
  o << n << '\n' << "test\n";
  for (int i = 0; i < n; ++i)
    o << type[i] << '\t' << pos[3 * (size_t)i] << '\t' << pos[3 * (size_t)i + 1] << '\t'
      << pos[3 * (size_t)i + 2] << '\n';
  f << o.str();
  return f.fail() ? 11 : 0;
}

}  // namespace smd
