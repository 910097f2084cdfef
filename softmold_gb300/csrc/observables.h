// Measurement files written by the `MD <name>` executable at each measure
// interval: dataExtraction<T,Blob>::compute (dataExtraction.h:827-1050,
// 1456-1488, 1509-1650), Kinetic<T>::output
// (include/algorithms/dataCollection.h:676-690) and the kinetic-energy
// histogram written by ~dataExtraction (dataExtraction.h:553-567).
//
// The potential energies are supplied by the caller (GPU reductions in the
// product, CPU sums in the oracle); everything else is computed here from the
// state the caller passes in, with the reference's formulas and output format.
#pragma once

#include <string>
#include <vector>

#include "mpd_io.h"

namespace smd {

// Aggregates of one measurement, from which the .dat lines are written: the
// host computes them from the state it holds (the oracle), the device from its
// own arrays (the GPU driver reads back only these).
struct Measurement {
  double kinetic = 0;                      // sum v^2/2 (Kinetic::compute)
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // smallest and largest coordinate per axis
  double lbond = 0;                        // sum of BOND residue bond lengths
  int n_bond = 0;
  double cos_bend = 0, l_bend0 = 0, l_bend1 = 0;  // BEND residue sums
  int n_bend = 0;
  bool msd = false;                        // diffusion started: write a meanSquareDisplacement_ line
  std::vector<double> msd_sum;             // per molecule: sum of squared displacements of its entries
};

// Bead entries whose displacements meanSquareDisplacement_ averages, per
// molecule in file order (dataExtraction.h:1524-1650): both beads of every
// BOND, the three of every BEND, every bead of every CHAIN block, each bead
// of a BEAD or NANOCORE residue; a bead listed twice counts twice.  Other
// molecule types have no entries (no column).  offsets has nMolecules + 1
// entries.
void msd_groups(const MpdSystem& sys, std::vector<int>& offsets, std::vector<int>& beads);

// Kinetic-energy bins of 1e-4 the histogram holds at most (energies below
// 6,710.8864 per bead), as the device measurement does.
constexpr int kMaxKeBins = 1 << 26;

class Observables {
 public:
  explicit Observables(const std::string& name) : name_(name) {}

  // One measurement from the state.  pos/vel: N*3 (current state), abs_pos:
  // unwrapped positions (may be null: no diffusion tracking and no
  // kinetic-energy histogram), time: current time.  pot: total potential
  // (pair + bonded + BEAD); bead_pot: BEAD part; n_bead_res: number of BEAD
  // residues.  Returns nonzero, writing nothing, when a bead's kinetic energy
  // lies beyond the histogram's kMaxKeBins bins (a run that has blown up).
  int compute(const MpdSystem& sys, double time, const double* pos, const double* vel,
               const double* abs_pos, double pot, double bead_pot, int n_bead_res);

  // The aggregates compute() writes from (and the kinetic-energy histogram
  // update when abs_pos is given); nonzero as compute().
  int aggregate(const MpdSystem& sys, const double* pos, const double* vel, const double* abs_pos,
                 Measurement& m);

  // Appends the measurement's lines to the .dat files.
  void write(const MpdSystem& sys, double time, double pot, double bead_pot, int n_bead_res,
             const Measurement& m);

  // dataExtraction::startDiffusion (dataExtraction.h:790-804).
  void start_diffusion(const MpdSystem& sys, const double* abs_pos);
  bool diffusion_started() const { return !msd_start_.empty(); }

  // The per-bead kinetic-energy histogram in bins of 1e-4 (its counts so far).
  std::vector<long>& ke_histogram() { return ke_hist_; }

  // Writes kEnergyDensity_<name>.dat (dataExtraction.h:553-567).
  void finish();

 private:
  void append(const std::string& prefix, const std::string& line);
  std::string name_;
  std::vector<long> ke_hist_;
  std::vector<double> msd_start_;
  std::vector<int> msd_off_, msd_beads_;
};

}  // namespace smd
