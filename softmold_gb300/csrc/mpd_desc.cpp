#include "mpd_desc.h"

#include <cmath>
#include <exception>
#include <initializer_list>
#include <memory>

namespace smd {

void set_last_error(const std::string& msg);

namespace {

// Terms of one external-field residue, in the order the reference applies
// them (kind = the molecule type; 8 constants each):
//   BOUNDARY (Blob::doBoundaryForce, include/system.h:2335-2349): one term per
//     bead, constants {dim, centre, -, k};
//   FLOATING_BASE (doFloatingBaseForce, :2403-2422): one term per bead, the 6
//     constants of the bead's type, then the residue's first constant (the
//     potential's z offset, doFloatingBasePotential :2437);
//   ZTORQUE (doZTorqueForce, :2626-2664): one term per bond (l, l+1) of each
//     chain but its last, constants {a, b, c, z0};
//   ZPOWERPOTENTIAL (doZPowerForce, :2693-2716): one term per bead of each
//     {start, count} block, constants {c0, c1};
//   BALL (doBallForce, :1937-1971): one term per bond (the residue's first
//     bond's first bead, this bond's second), constants {r0, k, this bond's
//     first} (the potential, doBallPotential :2750-2779, takes each bond's
//     own first).
void field_terms(const Molecule& m, const std::vector<int>& type, std::vector<int>& idx, std::vector<double>& cs) {
  auto push = [&](int a, int b, std::initializer_list<double> c) {
    idx.insert(idx.end(), {m.type, a, b});
    std::vector<double> v(c);
    v.resize(8, 0.0);
    cs.insert(cs.end(), v.begin(), v.end());
  };
  const std::vector<double>& C = m.constants;
  for (const auto& b : m.bonds) {
    if (m.type == MOL_BOUNDARY) {
      push(b[0], -1, {C[0], C[1], C[2], C[3]});
    } else if (m.type == MOL_FLOATING_BASE) {
      const double* t = C.data() + 6 * type[b[0]];
      push(b[0], -1, {t[0], t[1], t[2], t[3], t[4], t[5], C[0]});
    } else if (m.type == MOL_ZPOWERPOTENTIAL) {
      for (int k = b[0]; k < b[0] + b[1]; ++k) push(k, -1, {C[0], C[1]});
    } else if (m.type == MOL_BALL) {
      push(m.bonds[0][0], b[1], {C[0], C[1], (double)b[0]});
    } else {
      for (int k = b[0]; k < b[0] + b[2] * b[1]; k += b[2])
        for (int l = k; l < k + b[2] - 2; ++l) push(l, l + 1, {C[0], C[1], C[2], C[3]});
    }
  }
}

}  // namespace

int mpd_residues(const MpdSystem& S, MpdResidues& r, std::string& err) {
  bool sphere = false;
  for (const Molecule& m : S.mol) {
    if (m.type == MOL_CHAIN) {
      for (const auto& b : m.bonds) {
        r.blocks.insert(r.blocks.end(), {b[0], b[1], b[2]});
        r.chain_consts.insert(r.chain_consts.end(), m.constants.begin(), m.constants.begin() + 4);
      }
    } else if (m.type == MOL_BOND) {
      for (const auto& b : m.bonds) {
        r.bond_idx.insert(r.bond_idx.end(), {b[0], b[1]});
        r.bond_c.insert(r.bond_c.end(), m.constants.begin(), m.constants.begin() + 2);
      }
    } else if (m.type == MOL_BEND) {
      for (const auto& b : m.bonds) {
        r.bend_idx.insert(r.bend_idx.end(), {b[0], b[1], b[2]});
        r.bend_c.insert(r.bend_c.end(), m.constants.begin(), m.constants.begin() + 2);
      }
    } else if (m.type == MOL_BEAD || m.type == MOL_NANOCORE) {
      if (sphere) {
        err = "Error(MD): more than one BEAD or NANOCORE residue is not supported on the GPU step";
        return 1;
      }
      sphere = true;
      for (const auto& b : m.bonds) r.sphere_idx.push_back(b[0]);
      r.sphere_consts = m.constants;
      r.nanocore = (m.type == MOL_NANOCORE);
      ++r.n_bead_res;
    } else if (m.type == MOL_BOUNDARY || m.type == MOL_FLOATING_BASE || m.type == MOL_ZTORQUE ||
               m.type == MOL_ZPOWERPOTENTIAL || m.type == MOL_BALL) {
      field_terms(m, S.type, r.field_idx, r.field_c);
    } else if (m.type != MOL_SOLID) {
      err = "Error(MD): molecule type " + std::to_string(m.type) +
            " is not supported on the GPU step (supported: CHAIN, BOND, BEND, BEAD, NANOCORE, "
            "BOUNDARY, FLOATING_BASE, ZTORQUE, ZPOWERPOTENTIAL, BALL)";
      return 1;
    }
  }
  r.gamma = S.gamma;
  if (!(S.gamma > 0)) {
    if (!S.present[CMD_GAMMATYPE] || S.gammaType.empty()) {
      err = "Error(main): No gamma available!";
      return 2;
    }
    r.gamma = S.gammaType[0];  // the reference applies entry 0 to every bead
    r.per_type_gamma = true;
  }
  return 0;
}

void mpd_descriptor(const MpdSystem& S, const MpdResidues& r, smd_system_desc& d) {
  d = smd_system_desc{};
  d.n = S.nParticles;
  d.n_types = S.nTypes;
  d.pos = S.pos.data();
  d.vel = S.vel.data();
  d.type = S.type.data();
  for (int k = 0; k < 3; ++k) d.box[k] = S.size[k];
  d.cutoff = S.cutoff;
  d.fconst = S.twoBodyFconst.data();
  d.uconst = S.twoBodyUconst.data();
  d.n_chain_blocks = (int)r.blocks.size() / 3;
  d.chain_blocks = r.blocks.data();
  d.chain_consts = r.chain_consts.data();
  d.n_spheres = (int)r.sphere_idx.size();
  d.sphere_index = r.sphere_idx.data();
  d.sphere_consts = r.sphere_consts.empty() ? nullptr : r.sphere_consts.data();
  d.sphere_nanocore = r.nanocore ? 1 : 0;
  d.n_bonds = (int)r.bond_idx.size() / 2;
  d.bonds = r.bond_idx.data();
  d.bond_consts = r.bond_c.data();
  d.n_bends = (int)r.bend_idx.size() / 3;
  d.bends = r.bend_idx.data();
  d.bend_consts = r.bend_c.data();
  d.n_fields = (int)r.field_idx.size() / 3;
  d.fields = r.field_idx.data();
  d.field_consts = r.field_c.data();
  d.dt = S.deltaT;
  d.gamma = r.gamma;
  d.temperature = S.initialTemp;
  d.seed = (uint32_t)S.seed;
  d.tension = S.tension;
  d.delta_lxy = S.deltaLXY;
  d.resize_rate = 8;
  // (a deltaT the library refuses gives step 0 here)
  const double first = S.initialTime / S.deltaT + 0.0000001;
  d.first_step = (S.deltaT > 0 && std::fabs(first) < 2147483647.0) ? int(first) : 0;
}

}  // namespace smd

namespace {
struct LoadedMpd {
  smd::MpdSystem S;
  smd::MpdResidues r;
};

int load_mpd(const char* path, smd_system_desc* desc, smd_mpd_run* run, void** owner) {
  std::unique_ptr<LoadedMpd> L(new LoadedMpd);
  std::string err;
  if (int rc = smd::mpd_read_file(path, L->S, err)) {
    smd::set_last_error(err);
    return rc;
  }
  if (int rc = smd::mpd_residues(L->S, L->r, err)) {
    smd::set_last_error(err);
    return 10 + rc;
  }
  smd::mpd_descriptor(L->S, L->r, *desc);
  if (run) {
    const smd::MpdSystem& S = L->S;
    run->initial_time = S.initialTime;
    run->final_time = S.finalTime;
    run->store_interval = S.storeInterval;
    run->measure_interval = S.measureInterval;
    run->initial_temp = S.initialTemp;
    run->final_temp = S.finalTemp;
    run->temp_step_interval = S.tempStepInterval;
    run->n_bead_residues = L->r.n_bead_res;
    run->per_type_gamma = L->r.per_type_gamma ? 1 : 0;
  }
  *owner = L.release();
  return 0;
}

}  // namespace

extern "C" int smd_mpd_load(const char* path, smd_system_desc* desc, smd_mpd_run* run, void** owner) {
  if (!path || !desc || !owner) return 1;
  *owner = nullptr;
  // the reader refuses counts its file cannot hold; what it allocates for the
  // rest comes back as error code 9 rather than an exception through the ABI
  try {
    return load_mpd(path, desc, run, owner);
  } catch (const std::exception& e) {
    smd::set_last_error(std::string("smd_mpd_load: ") + e.what());
    return 9;
  }
}

extern "C" void smd_mpd_free(void* owner) { delete static_cast<LoadedMpd*>(owner); }
