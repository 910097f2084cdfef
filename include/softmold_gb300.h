/*
 * softmold_gb300 — C ABI of the GB300 implicit-solvent membrane MD step.
 *
 * The reference (SoftMold) has no FFI layer for this path: its `MD <name>`
 * driver (MD.cpp:72-755) calls C++ templates in-process.  Each entry point
 * below names the reference call it replaces.  All calls take and return plain
 * host pointers and sizes; the library owns all device memory.  Status codes:
 * 0 = OK, nonzero = error, with the message available from smd_last_error().
 * Handles are not thread-safe; use one handle per host thread / stream.
 *
 * Layout conventions: per-bead vectors are AoS double x,y,z (n*3), bead order
 * is the order of the .mpd file; constant tables are the reference's flat
 * layouts (twoBodyFconst/Uconst: 6 doubles per ordered type pair, BEAD: 22).
 */
#ifndef SOFTMOLD_GB300_H
#define SOFTMOLD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SMD_ABI_VERSION 1

/* Arithmetic of the pair and bonded forces. */
enum smd_precision {
  SMD_PLAIN_FP64 = 0, /* every force term in FP64, FP64 accumulation */
  SMD_MIXED = 1       /* FP32 force arithmetic, int64 fixed-point accumulation,
                         FP64 integrator, barostat and energy sums */
};

/* One membrane system (one replica).  Mirrors the Blob<double> fields the
 * hot path reads (include/system.h:247-290). */
typedef struct smd_system_desc {
  int n;                        /* beads (nParticles) */
  int n_types;                  /* nTypes */
  const double* pos;            /* n*3, each coordinate in [0, box] */
  const double* vel;            /* n*3 */
  const int* type;              /* n */
  double box[3];                /* size */
  double cutoff;                /* rc */
  const double* fconst;         /* 6*n_types^2 twoBodyFconst */
  const double* uconst;         /* 6*n_types^2 twoBodyUconst */
  int n_chain_blocks;           /* CHAIN residue blocks */
  const int* chain_blocks;      /* n_chain_blocks*3: start, nChains, length */
  const double* chain_consts;   /* n_chain_blocks*4: l0, kbond, abend, kbend */
  int n_spheres;                /* beads of one BEAD residue (0 = none, at most 256); up to 20 a
                                   sphere's force leaves out the other spheres, above 20 it takes
                                   them (Blob::doBeadForce's two branches, system.h:2104-2210) */
  const int* sphere_index;      /* n_spheres bead indices */
  const double* sphere_consts;  /* 22*n_types^2 BEAD constants */
  double dt;                    /* deltaT */
  double gamma;                 /* Langevin friction */
  double temperature;           /* kT (initialTemp) */
  uint32_t seed;                /* .mpd seed: barostat trials and Langevin noise */
  double tension;               /* constant-tension barostat target */
  double delta_lxy;             /* MC box-move amplitude, 0 = barostat off */
  int resize_rate;              /* MC move every resize_rate steps (MD.cpp:67: 8) */
  int first_step;               /* loop index of the first step (initialTime/deltaT) */
  double skin;                  /* Verlet-list skin in sigma (<=0: default 0.5) */
  int n_bonds;                  /* terms of BOND residues (Blob::doBondForce) */
  const int* bonds;             /* n_bonds*2 bead indices: first, second */
  const double* bond_consts;    /* n_bonds*2: l0, k of each term's residue */
  int n_bends;                  /* terms of BEND residues (Blob::doBendForce) */
  const int* bends;             /* n_bends*3 bead indices: first, second, third */
  const double* bend_consts;    /* n_bends*2: a, k of each term's residue */
  int n_fields;                 /* terms of external-field residues, in the order the reference applies them */
  const int* fields;            /* n_fields*3: kind (the .mpd molecule type: 11 BOUNDARY, 15 FLOATING_BASE,
                                   16 ZTORQUE, 17 ZPOWERPOTENTIAL, 19 BALL), first bead, second bead
                                   (ZTORQUE, BALL; else -1) */
  const double* field_consts;   /* n_fields*8: BOUNDARY {dim, centre, -, k} (Blob::doBoundaryForce);
                                   FLOATING_BASE the 6 constants of the bead's type, then the residue's
                                   first constant (doFloatingBaseForce); ZTORQUE {a, b, c, z0} for one
                                   bond (l, l+1) (doZTorqueForce); ZPOWERPOTENTIAL {c0, c1} (doZPowerForce);
                                   BALL {r0, k, the bond's own first bead} with first = the residue's
                                   first bond's first bead (doBallForce / doBallPotential) */
  int sphere_nanocore;          /* 1: the sphere beads form a NANOCORE residue (Blob::doNanoCoreForce):
                                   sphere_consts holds 22 constants per bead, each bead acts on every
                                   other bead (other cores included) with its own row and has the mass
                                   4 pi R^2 of its own radius, divided once a step
                                   (MD.cpp:291-303, 495-507); no sphere-sphere term,
                                   no size-change term */
} smd_system_desc;

typedef struct smd_system smd_system;

typedef struct smd_energy {
  double pair;     /* CellOpt::computePotential */
  double bonded;   /* Blob::doChainPotential, doBondPotential, doBendPotential and the
                      external-field potentials (doBoundaryPotential, doFloatingBasePotential,
                      doZTorquePotential, doZPowerPotential, doBallPotential) */
  double sphere;   /* Blob::doBeadPotential */
  double kinetic;  /* Kinetic::compute: sum v^2/2 */
} smd_energy;

typedef struct smd_mc_stats {
  long trials;
  long accepted;
  double last_dU;  /* last trial's potential difference incl. tension term */
} smd_mc_stats;

/* Last error message of the calling thread; returns its length. */
int smd_last_error(char* buf, size_t len);

/* Number of visible CUDA devices (0 when none). */
int smd_device_count(void);

/* Builds the device state for one system (replaces the Verlet / Langevin /
 * CellOpt constructors, MD.cpp:124-154).  precision: enum smd_precision. */
int smd_create(const smd_system_desc* desc, int precision, smd_system** out);

/* Builds n independent replicas that advance together in the same launches
 * with per-replica offsets, boxes, seeds, tensions and barostat decisions. */
int smd_create_batch(const smd_system_desc* descs, int n, int precision, smd_system** out);

void smd_destroy(smd_system* h);

/* Runs later work on this CUDA stream (cudaStream_t; NULL = library stream). */
int smd_set_stream(smd_system* h, void* cuda_stream);

/* Copies all beads' state, replicas concatenated, in input order, xyz per
 * bead (Blob::getPositions / getVelocities).  Either pointer may be NULL.
 * The permutation to the device's cell order runs on the device, so each
 * array is one contiguous host copy (fastest from pinned memory).  Setting
 * positions rebuilds the Verlet list, growing it if the new configuration
 * is denser. */
int smd_get_state(smd_system* h, double* pos, double* vel);
int smd_set_state(smd_system* h, const double* pos, const double* vel);
int smd_get_box(smd_system* h, int replica, double box[3]);
/* Sets a replica's box without moving the beads (Blob::setSize,
 * include/system.h:4436-4444); positions must lie inside the new box. */
int smd_set_box(smd_system* h, int replica, const double box[3]);

/* Conservative forces at the current positions, no Langevin term:
 * CellOpt::computeForce + Blob::doChainForce (+ doBeadForce)
 * (include/algorithms/cellOpt.h:712-926, include/system.h:1782-1866,2043-2212). */
int smd_compute_forces(smd_system* h, double* force_out);

/* Non-bonded forces only (CellOpt::computeForce). */
int smd_compute_pair_forces(smd_system* h, double* force_out);

/* Energies at the current state, per replica (energies[n_replicas]):
 * CellOpt::computePotential, Blob::doChainPotential, doBeadPotential and
 * Kinetic::compute (cellOpt.h:928-1041, system.h:2487-2568, 2936-3074). */
int smd_compute_energy(smd_system* h, smd_energy* energies);

/* U(x) - U(s*x) summed over pairs within rc, CHAIN and BEAD terms, for an
 * affine box scale s (CellOpt::computeDPotential + Blob::do*DPotential,
 * cellOpt.h:1043-1180, system.h:3280-3384). One value per replica. */
int smd_compute_dU(smd_system* h, const double scale[3], double* dU);

/* CellOpt cell key of every bead for the reference grid nCells=int(L/rc)
 * (cellOpt.h:532-555), computed on the GPU. */
int smd_cell_keys(smd_system* h, int* keys);

/* Unordered pairs (i<j, file order) with r < rc taken from the GPU Verlet
 * list; writes at most cap pairs and stores the total count. */
int smd_pair_list(smd_system* h, int* pairs, size_t cap, size_t* count);

/* Start-up of MD.cpp:186-308: initial build, forces and thermostat, then the
 * restart half-kick when initial_time != 0 (do_second), then the first
 * half-kick and drift of the first loop step.  If energy_out is not NULL the
 * energies at the initial positions and velocities are stored there before
 * any update (the t = 0 measurement). */
int smd_prepare(smd_system* h, int do_second, smd_energy* energy_out);

/* Advances `steps` iterations of the MD.cpp:335-729 loop body: thermostat,
 * pair and bonded forces, second half-kick, the MC box move on every
 * resize_rate-th step, and the next step's first half-kick and drift.
 * flags: SMD_STOP_AT_MEASURE stops the last iteration after its second
 * half-kick so the caller can read the measured state (the next smd_advance
 * call, steps may be 0, completes that iteration); SMD_ASYNC returns without
 * waiting for the device (errors surface at the next synchronising call or
 * smd_sync). */
#define SMD_STOP_AT_MEASURE 1
#define SMD_ASYNC 2
int smd_advance(smd_system* h, int steps, int flags);

/* Autotuner of the mixed form's launch configuration (no reference
 * counterpart): times the Verlet-list build variants (flat stencil with 128 or
 * 256 threads per cell, octant-filtered) and the pair pass at 4, 8 and 16
 * lanes per bead on the handle's state, and keeps the fastest of each; every
 * choice gives bitwise the same trajectory.  smd_advance runs it once per
 * system shape, at its first call after the handle has run 256 steps (the
 * running membrane, not its start configuration; environment SMD_AUTOTUNE=0
 * turns that off); force = 1 re-times.  Reports the choice
 * (lanes: 4/8/16; list_kernel: 0 flat-128, 1 flat-256, 2 octant) and, in
 * ms[6] if not NULL, the best times of the three list variants and of the
 * three lane counts.  The plain form keeps its fixed configuration. */
int smd_autotune(smd_system* h, int force, int* lanes, int* list_kernel, float* ms);

/* Sets the launch configuration the autotuner would choose (lanes 4, 8 or
 * 16; list_kernel 0, 1 or 2) and marks the handle tuned. */
int smd_set_tuning(smd_system* h, int lanes, int list_kernel);

/* Launch mode of smd_advance: on = 1 (default) runs each barostat period as
 * one CUDA graph whose list builds are conditional nodes; on = 0 launches the
 * same kernels one by one (profilers that cannot see kernel nodes inside
 * graphs with conditional nodes still see each kernel).  No reference
 * counterpart: the reference launches nothing. */
int smd_use_graphs(smd_system* h, int on);

/* Waits for the handle's stream and reports any device-side error. */
int smd_sync(smd_system* h);

/* Barostat statistics of a replica. */
int smd_mc_stats_get(smd_system* h, int replica, smd_mc_stats* out);

/* Box-move history of a replica: for trials [start, start+max) the x/y
 * fluctuation drawn (MD.cpp:595) and whether it was accepted.  Returns the
 * number of entries written, or a negative value on error. */
long smd_mc_log(smd_system* h, int replica, long start, long max, double* fluct, int* accepted);

/* Changes the thermostat temperature (the tempStepInterval ramp,
 * MD.cpp:369-371).  update_sigma = 0 keeps the noise amplitude, as the
 * reference does for per-type gammas (langevin.h:235-246). replica -1 = all. */
int smd_set_temperature(smd_system* h, int replica, double kT, int update_sigma);

/* Langevin noise from the caller for the next force evaluation: psi[n*3] in
 * [-1,1), bead order, used once instead of the counter-based generator.
 * Lets a test drive the device step with the reference's MT19937 stream. */
int smd_set_noise_once(smd_system* h, const double* psi);

/* Per-launch CUDA-event timing of the fused step kernel (on = 1).  While on,
 * every step-kernel launch is bracketed by events on the handle's stream. */
int smd_profile(smd_system* h, int on);

/* Accumulated device time (ms) and launch count of the fused step kernel
 * since profiling was switched on, and the total number of kernel launches
 * the handle has issued. */
int smd_last_timing(smd_system* h, double* step_kernel_ms, long* step_kernel_launches, long* total_launches);

/* Number of Verlet-list rebuilds so far. */
long smd_rebuild_count(smd_system* h);

/* Largest bead displacement from its list-build position seen by the last
 * step, and the list-distance slack used by accepted box moves since the
 * build (both in sigma; the list is rebuilt when their sum exceeds skin/2). */
int smd_list_state(smd_system* h, double* max_disp, double* slack);

/* Measurement of one measure step on the device (dataExtraction::compute,
 * dataExtraction.h:827-1050, 1456-1650, and Kinetic::compute,
 * include/algorithms/dataCollection.h:666-674), for handles stopped at a
 * measure step (smd_advance with SMD_STOP_AT_MEASURE): the reductions the
 * .dat files need, so that only these few numbers cross to the host.
 * Single-system handles. */
typedef struct smd_measurement {
  double kinetic;          /* sum v^2/2 (kinetic_) */
  double lo[3], hi[3];     /* smallest and largest coordinate per axis (flicker_) */
  double bond_length_sum;  /* BOND residue bond lengths (lBond_) */
  int n_bond;
  double bend_cos_sum, bend_len0_sum, bend_len1_sum;  /* BEND residues (bend_) */
  int n_bend;
  int msd;                 /* 1: msd_sum holds the groups' sums (diffusion tracking on) */
} smd_measurement;

/* Fills *out and, while diffusion is tracked, msd_sum[n_groups] (may be NULL)
 * with each group's sum of squared displacements since smd_start_diffusion;
 * adds every bead's kinetic-energy bin int(0.5 v^2 / 1e-4)
 * (dataExtraction.h:1509-1519) to the run's histogram on the device. */
int smd_measure(smd_system* h, smd_measurement* out, double* msd_sum);

/* The kinetic-energy histogram smd_measure has accumulated (the
 * kEnergyDensity_ file written at the end of a run, dataExtraction.h:553-567):
 * counts of bins of 1e-4 from 0; writes at most cap bins and stores the
 * number of bins (the last non-empty bin + 1) in *n_bins. */
int smd_ke_histogram(smd_system* h, long* counts, size_t cap, size_t* n_bins);

/* dataExtraction::startDiffusion (dataExtraction.h:790-804, called by MD.cpp
 * at the first measure step after 100 tau): from now on every drift adds
 * v dt to each bead's displacement (nonzero types), as Verlet::first advances
 * the absolute positions aP (include/algorithms/verlet.h:317-326); box moves
 * do not rescale it (MD.cpp:555).  Calling it again restarts from zero. */
int smd_start_diffusion(smd_system* h);

/* The groups of meanSquareDisplacement_ (dataExtraction.h:1524-1650): group g
 * averages the displacements of beads[offsets[g] .. offsets[g+1]) (file
 * order; a bead may appear more than once, as the reference counts it). */
int smd_set_msd_groups(smd_system* h, int n_groups, const int* offsets, const int* beads);

/* Runs the synthetic generators (restating generate/liposome.cpp,
 * generate/bilayer.cpp and generate/continuumSphereAndLiposome.cpp) and
 * writes <path>.  An allocation that fails returns 9 (message in
 * smd_last_error). */
int smd_synth_vesicle(const char* path, int seed, int n_lipids, double areal_density, double box);
int smd_synth_bilayer(const char* path, int seed, int n_lipids, double areal_density, double zsize,
                      double delta_lxy, double tension);
int smd_synth_vesicle_sphere(const char* path, int seed, int n_lipids, double areal_density,
                             double box, double sphere_radius, double head_umin, double head_umax,
                             double gap, double other_umax);

/* Non-bonded forces for callers that cannot allocate device memory (for
 * example code running while another framework owns the device memory
 * through its own pool, or a loop that must not take cudaMalloc's implicit
 * device-wide synchronisation).  No counterpart in the reference: it is the
 * FP64 non-bonded force of smd_compute_pair_forces for device-resident
 * inputs, with its cell-list scratch in a fixed array inside the library
 * instead of allocated memory.  d_pos (n*3), d_type (n), d_fconst
 * (6*n_types^2) and d_force (n*3, overwritten) are device pointers owned by
 * the caller; work is queued on `stream` (a cudaStream_t, NULL = default) and
 * not waited for.  At most SMD_STATIC_MAX_BEADS beads and
 * SMD_STATIC_MAX_CELLS cells (int(L/rc) per axis); larger inputs, and box
 * edges that are not finite and positive, are rejected.  Positions must be
 * wrapped into [0, L] for the forces to be the reference's, and types must
 * lie in [0, n_types).  The device arrays are not checked on the host, but
 * no value in them makes a kernel access memory outside the caller's arrays
 * and the scratch: cell indices are clamped into the grid and types are
 * range-checked before the table lookup; a bead whose position is not
 * finite, or whose type or a neighbour's type within rc is outside
 * [0, n_types), gets a NaN force.  Calls share the scratch: calls that
 * overlap on the GPU race.  The first call on a device looks up the scratch
 * address; make it before any stream capture, and do not call this entry
 * point on a device again after cudaDeviceReset of that device. */
#define SMD_STATIC_MAX_BEADS 32768
#define SMD_STATIC_MAX_CELLS 32768
int smd_pair_forces_static(const double* d_pos, const int* d_type, int n, const double box[3], double cutoff,
                           int n_types, const double* d_fconst, double* d_force, void* stream);

/* Gradient of a time average with respect to potential constants (no
 * reference counterpart: the reference computes no derivatives).  From the
 * handle's current state (x_1, h_1), h the half-step velocity, the observable
 * J = (1/T) sum_{n=1..T} U(x_n), U the pair + CHAIN potential at the
 * positions where step n evaluates its forces, is differentiated through T
 * loop steps (MD.cpp:335-729) with the Langevin noise fixed by its seed and
 * the box fixed (barostat off).  The forward pass stores the state every
 * checkpoint_every steps; the backward pass recomputes each segment and runs
 * the discrete adjoint of the step (Hessian-vector products over the Verlet
 * list, FP32 pair terms in the mixed form, FP64 accumulation).  Parameters:
 * Umin of the type pair umin_types (both ordered table rows,
 * include/potentials/laradjiRevalee.h:84-152), and kbond and kbend, the CHAIN
 * constants 1 and 3 of every CHAIN residue.  Afterwards the handle holds the
 * state after the T steps, as smd_advance(h, T, 0) leaves it.  Single-system
 * handles without BEAD residues. */
typedef struct smd_adjoint_spec {
  int steps;             /* T >= 1 */
  int checkpoint_every;  /* >= 1 */
  int umin_types[2];     /* type pair (a, b) of the Umin parameter */
  int segment_local;     /* 0: the exact derivative of J; 1: each segment's
                            terms differentiated through that segment only
                            (the adjoint state restarts at every checkpoint),
                            which stays bounded where the exact derivative of
                            a long window grows exponentially (chaotic runs) */
} smd_adjoint_spec;

typedef struct smd_adjoint_result {
  double mean_potential;       /* J */
  double grad[3];              /* dJ/dUmin(a,b), dJ/dkbond, dJ/dkbend */
  double mean_area_per_lipid;  /* box_x box_y / (CHAIN molecules / 2) */
  double grad_area[3];         /* 0: the box does not depend on the constants here */
} smd_adjoint_result;

int smd_adjoint(smd_system* h, const smd_adjoint_spec* spec, smd_adjoint_result* out);

/* K w with K = dF/dx the Jacobian of the conservative pair + CHAIN forces at
 * the current positions (minus the Hessian of U), w and kw n*3 in file order.
 * The product the adjoint step uses; exposed to check it against finite
 * differences of the forces. */
int smd_hessian_vector(smd_system* h, const double* w, double* kw);

/* Rewrites the .mpd at in_path with new positions, velocities, box and
 * initialTime into out_path (the store of MD.cpp:373-377).  A file the reader
 * refuses returns its nonzero status, an allocation that fails 9 (message in
 * smd_last_error). */
int smd_mpd_update_state(const char* in_path, const char* out_path, const double* pos, const double* vel,
                         const double box[3], double time);

/* Run settings of an .mpd that the descriptor does not carry. */
typedef struct smd_mpd_run {
  double initial_time, final_time, store_interval, measure_interval;
  double initial_temp, final_temp, temp_step_interval;
  int n_bead_residues;  /* BEAD and NANOCORE residues (beadPotential_ output) */
  int per_type_gamma;   /* 1: gamma came from gammaType (entry 0 applies to every bead) */
} smd_mpd_run;

/* Reads <path> with the library's .mpd reader (Blob::input restated,
 * include/system.h:589-1314, through Script::read, scriptFormat.h:79-94) and
 * fills *desc with the system and every residue the device step runs,
 * expanded as the `MD` executable expands them (CHAIN blocks, BOND and BEND
 * terms, one BEAD or NANOCORE residue, external-field terms); run may be
 * NULL.  The descriptor's arrays belong to *owner until smd_mpd_free(*owner).
 * A residue type the device step does not run is refused (status 11), as is
 * a file without gamma (12).  The reader refuses a negative count, or one
 * whose entries the file does not hold, before allocating for it; an
 * allocation that fails returns 9.  Messages are in smd_last_error. */
int smd_mpd_load(const char* path, smd_system_desc* desc, smd_mpd_run* run, void** owner);
void smd_mpd_free(void* owner);

/* Reads <name>.mpd and runs it exactly as `MD <name>` would, writing the
 * same .mpd / .xyz / .dat files (MD.cpp:72-755).  precision: smd_precision. */
int smd_md_main(const char* name, int precision);

#ifdef __cplusplus
}
#endif
#endif /* SOFTMOLD_GB300_H */
