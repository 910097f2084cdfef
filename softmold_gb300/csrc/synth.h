// Seeded synthetic membrane inputs in the reference generators' terms.
//
// Restates the geometry of models/lipidModels.h liposome() (:1313-1469) and
// bilayer() (:1747-1924), models/nanoModels.h continuumSphere() (:120-175),
// the constant tables of include/potentials/laradjiRevalee.h:84-152 and
// laradjiSpangler.h:186-270, and the run settings of generate/liposome.cpp,
// generate/bilayer.cpp and generate/continuumSphereAndLiposome.cpp.  With the
// reference generators' arguments the .mpd written here is byte-identical to
// theirs; the extra knobs (box size, z height, steps) select the benchmark
// workloads.
#pragma once
#include <string>
#include <vector>

#include "mpd_io.h"

namespace smd {

// Bead types (generate/include.h:28-35, include/MD.h:20-27).
constexpr int kHead = 2, kTail = 3, kAnchor = 5;

// Non-bonded force / potential constant tables for an nT x nT Umax/Umin grid
// (index i + j*nT), rc and rm.
std::vector<double> laradji_revalee_fc(const std::vector<double>& Umax, const std::vector<double>& Umin,
                                       double rc, double rm);
std::vector<double> laradji_revalee_pc(const std::vector<double>& Umax, const std::vector<double>& Umin,
                                       double rc, double rm);
// One 22-constant continuum-sphere row (laradjiSpanglerFCrow).
std::vector<double> laradji_spangler_row(double rc, double rm, double rad, double density, double Umax,
                                         double Umin);

// generate/liposome.cpp: name seed nLipids arealDensity, box edge `box`
// (the reference uses 400), vesicle centred.
MpdSystem synth_vesicle(int seed, int nLipids, double density, double box);
// generate/bilayer.cpp with no anchors: z size `zsize` (the reference uses 40).
MpdSystem synth_bilayer(int seed, int nLipids, double density, double zsize, double deltaLXY,
                        double tension);
// Adds one continuum sphere (BEAD residue) of radius R at pos with the
// continuumSphereAndLiposome tables (head well depth uminHead).
void add_continuum_sphere(MpdSystem& s, const double pos[3], double R, double uminHead, double umaxHead,
                          double umaxOther,
                          int beadType);

}  // namespace smd
