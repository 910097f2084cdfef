// Residues of an .mpd system as the device step takes them: the one expansion
// of the .mpd's molecule list into the descriptor of smd_create, shared by the
// `MD` executable and smd_mpd_load (the readers of the Python mirror, the
// tests and the bench go through it too).
#pragma once

#include <string>
#include <vector>

#include "../../include/softmold_gb300.h"
#include "mpd_io.h"

namespace smd {

struct MpdResidues {
  std::vector<int> blocks;          // CHAIN blocks: start, nChains, length
  std::vector<double> chain_consts; // 4 per block
  std::vector<int> sphere_idx;      // the beads of one BEAD or NANOCORE residue
  std::vector<double> sphere_consts;
  bool nanocore = false;
  int n_bead_res = 0;               // BEAD and NANOCORE residues (beadPotential_, dataExtraction.h:1031-1040)
  std::vector<int> bond_idx, bend_idx;
  std::vector<double> bond_c, bend_c;
  std::vector<int> field_idx;       // external-field terms: kind, first, second
  std::vector<double> field_c;      // 8 constants each
  double gamma = 0;                 // the Langevin friction the step applies
  bool per_type_gamma = false;      // taken from gammaType (entry 0, langevin.h:257)
};

// Expands the molecules of S.  Returns 0, or 1 with a message for a residue
// type the device step does not run, or 2 when the file gives no gamma (the
// reference's "No gamma available!", MD.cpp exits there with status 0).
int mpd_residues(const MpdSystem& S, MpdResidues& r, std::string& err);

// The descriptor of smd_create for S and its expanded residues (pointers into
// S and r, which must outlive it).
void mpd_descriptor(const MpdSystem& S, const MpdResidues& r, smd_system_desc& d);

}  // namespace smd
