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

class Observables {
 public:
  explicit Observables(const std::string& name) : name_(name) {}

  // One measurement.  pos/vel: N*3 (current state), abs_pos: unwrapped
  // positions (may be null: no diffusion tracking), time: current time.
  // pot: total potential (pair + bonded + BEAD); bead_pot: BEAD part;
  // n_bead_res: number of BEAD residues.
  void compute(const MpdSystem& sys, double time, const double* pos, const double* vel,
               const double* abs_pos, double pot, double bead_pot, int n_bead_res);

  // dataExtraction::startDiffusion (dataExtraction.h:790-804).
  void start_diffusion(const MpdSystem& sys, const double* abs_pos);
  bool diffusion_started() const { return !msd_start_.empty(); }

  // Writes kEnergyDensity_<name>.dat (dataExtraction.h:553-567).
  void finish();

 private:
  void append(const std::string& prefix, const std::string& line);
  std::string name_;
  std::vector<long> ke_hist_;
  std::vector<double> msd_start_;
};

}  // namespace smd
