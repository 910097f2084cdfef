// Host-only C ABI entries: the synthetic input generators.
#include <cmath>
#include <exception>
#include <string>

#include "../../include/softmold_gb300.h"
#include "mpd_io.h"
#include "synth.h"

namespace smd {
void set_last_error(const std::string& msg);
}

namespace {

// The generators and the state rewrite allocate from caller sizes and file
// counts: an allocation failure comes back as error code 9 with its message
// (smd_last_error), never as an exception through the C ABI.
template <typename F>
int no_throw(const char* what, F&& body) {
  try {
    return body();
  } catch (const std::exception& e) {
    smd::set_last_error(std::string(what) + ": " + e.what());
    return 9;
  }
}

}  // namespace

extern "C" {

int smd_synth_vesicle(const char* path, int seed, int n_lipids, double density, double box) {
  if (!path || n_lipids <= 0 || !(density > 0) || !(box > 0)) return 1;
  return no_throw("smd_synth_vesicle", [&] {
    std::string err;
    return smd::mpd_write_file(path, smd::synth_vesicle(seed, n_lipids, density, box), err);
  });
}

int smd_synth_bilayer(const char* path, int seed, int n_lipids, double density, double zsize, double delta_lxy,
                      double tension) {
  if (!path || n_lipids <= 0 || !(density > 0) || !(zsize > 0)) return 1;
  return no_throw("smd_synth_bilayer", [&] {
    std::string err;
    return smd::mpd_write_file(path, smd::synth_bilayer(seed, n_lipids, density, zsize, delta_lxy, tension), err);
  });
}

int smd_synth_vesicle_sphere(const char* path, int seed, int n_lipids, double density, double box,
                             double sphere_radius, double head_umin, double head_umax, double gap,
                             double other_umax) {
  if (!path || n_lipids <= 0 || !(density > 0) || !(box > 0) || !(sphere_radius > 1)) return 1;
  return no_throw("smd_synth_vesicle_sphere", [&] {
    smd::MpdSystem s = smd::synth_vesicle(seed, n_lipids, density, box);
    // sphere centred on the +z axis, its surface `gap` outside the outer heads
    // (outer head shell: radius + 5 bond lengths, models/lipidModels.h:1428-1431)
    const double R = std::sqrt(((double)n_lipids / density) / (4.0 * M_PI));
    const double c[3] = {box / 2.0, box / 2.0, box / 2.0 + R + 0.7 * 5 + gap + sphere_radius};
    smd::add_continuum_sphere(s, c, sphere_radius, head_umin, head_umax, other_umax, 4);
    std::string err;
    return smd::mpd_write_file(path, s, err);
  });
}

int smd_mpd_update_state(const char* in_path, const char* out_path, const double* pos, const double* vel,
                         const double box[3], double time) {
  if (!in_path || !out_path) return 1;
  return no_throw("smd_mpd_update_state", [&] {
    smd::MpdSystem s;
    std::string err;
    if (int rc = smd::mpd_read_file(in_path, s, err)) {
      smd::set_last_error(err);
      return rc;
    }
    const size_t n = 3 * (size_t)s.nParticles;
    if (pos) s.pos.assign(pos, pos + n);
    if (vel) s.vel.assign(vel, vel + n);
    if (box)
      for (int k = 0; k < 3; ++k) s.size[k] = box[k];
    s.initialTime = time;
    return smd::mpd_write_file(out_path, s, err);
  });
}

}  // extern "C"
