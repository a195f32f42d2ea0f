/*
 * azplugins_gb300.h -- C ABI of the GB300-native short-range force-and-integrate
 * path (cell list + neighbour list, azplugins pair and bond evaluators, Langevin /
 * Brownian dynamics in a flow field). Plain pointers, sizes and PODs only; every
 * device entry takes an explicit cudaStream_t (passed as void*), never allocates
 * inside a stream-ordered call, and returns an int status (0 = ok).
 *
 * Reference interfaces replaced (paths inside the azplugins tree):
 *   parameter structs   src/PairEvaluatorPerturbedLennardJones.h:25-66,
 *                       src/PairEvaluatorExpandedYukawa.h:23-53,
 *                       src/PairEvaluatorHertz.h:23-47,
 *                       src/PairEvaluatorColloid.h:23-57,
 *                       src/BondEvaluatorQuartic.h:28-82,
 *                       src/BondEvaluatorDoubleWell.h:28-61
 *   pair force driver   gpu_compute_pair_forces<Eval>, instantiated in
 *                       src/PotentialPairGPUKernel.cu.inc:25-28
 *   bond force driver   gpu_compute_bond_forces<Eval,2>, instantiated in
 *                       src/PotentialBondGPUKernel.cu.inc:25-29
 *   Langevin flow       gpu::langevin_flow_step1 / langevin_flow_step2<Flow>,
 *                       src/TwoStepLangevinFlowGPU.cuh:25-55
 *   Brownian flow       gpu::brownian_flow<Flow>, src/TwoStepBrownianFlowGPU.cuh:26-44
 *   flow fields         src/ConstantFlow.h:30-65, src/ParabolicFlow.h:51-98
 *   RNG stream ids      src/RNGIdentifiers.h:20-27
 *   harmonic barriers   HarmonicBarrierGPU<Evaluator>, src/HarmonicBarrierGPU.cuh:50-83
 *   wall potentials     gpu_compute_potential_external_forces<EvaluatorWalls<...>>,
 *                       src/PotentialExternalWallGPUKernel.cu.inc:26-30
 *   velocity fields     VelocityFieldComputeGPU<BinOp>, src/VelocityFieldComputeGPU.cuh:35-72;
 *                       VelocityComputeGPU, src/VelocityComputeGPU.cu:49-62
 */
#ifndef AZPLUGINS_GB300_H_
#define AZPLUGINS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AZP_ABI_VERSION 2

/* every entry point is exported; everything else in the library is hidden */
#if defined(__GNUC__)
#define AZP_API __attribute__((visibility("default")))
#else
#define AZP_API
#endif

/* ------------------------------------------------------------------ status */
enum azp_status {
    AZP_OK = 0,
    AZP_ERR_INVALID = -1,         /* bad argument */
    AZP_ERR_CUDA = -2,            /* a CUDA runtime call failed */
    AZP_ERR_NLIST_OVERFLOW = -3,  /* a particle has more neighbours than the list holds */
    AZP_ERR_BOND = -4,            /* a bond evaluator refused (r_0 == 0, r_1 == r_0) */
    AZP_ERR_BOX_TOO_SMALL = -5,   /* L < 2 (r_cut + r_buff) along a periodic axis */
    AZP_ERR_TIMEOUT = -6,         /* a bounded device wait gave up */
    AZP_ERR_NONFINITE = -7,       /* a non-finite position was produced */
    AZP_ERR_UNSUPPORTED = -8,     /* combination not built */
    AZP_ERR_CELL_OVERFLOW = -9,   /* internal cell list capacity exceeded */
    AZP_ERR_NO_DEVICE = -10,      /* no CUDA device visible */
    AZP_ERR_TOO_LARGE = -11       /* size above a fixed limit of the entry point */
};

/* device error word bits (azp_md_error / azp_err_word) */
#define AZP_EBIT_NLIST_OVERFLOW 0x1u
#define AZP_EBIT_BOND 0x2u
#define AZP_EBIT_NONFINITE 0x4u
#define AZP_EBIT_TIMEOUT 0x8u
#define AZP_EBIT_CELL_OVERFLOW 0x10u
#define AZP_EBIT_RANGE 0x20u          /* a value outside a fixed-point range */

/* ------------------------------------------------------------------ kinds */
enum azp_pair_kind {
    AZP_PAIR_PERTURBED_LJ = 0,     /* PairEvaluatorPerturbedLennardJones */
    AZP_PAIR_EXPANDED_YUKAWA = 1,  /* PairEvaluatorExpandedYukawa */
    AZP_PAIR_HERTZ = 2,            /* PairEvaluatorHertz */
    AZP_PAIR_COLLOID = 3,          /* PairEvaluatorColloid */
    AZP_PAIR_NUM_KINDS = 4,        /* kinds of azp_pair_forces */
    AZP_PAIR_DPD_GENERAL_WEIGHT = 4 /* DPDPairEvaluatorGeneralWeight: azp_dpd_forces and the engine */
};
enum azp_bond_kind {
    AZP_BOND_QUARTIC = 0,          /* BondEvaluatorQuartic */
    AZP_BOND_DOUBLE_WELL = 1,      /* BondEvaluatorDoubleWell */
    AZP_BOND_NUM_KINDS = 2,        /* kinds with the minimum-image displacement */
    AZP_BOND_IMAGE_HARMONIC = 2    /* ImagePotentialBondHarmonic (src/ImagePotentialBond.h): harmonic
                                      U = k/2 (r - r0)^2 on the image-unwrapped distance; azp_bond_forces
                                      (reads sys->image) and the engine (azp_md_config.bond_kind) */
};
/* HOOMD pair.Pair modes accepted by azplugins (src/pair.py:415) */
enum azp_shift_mode { AZP_MODE_NONE = 0, AZP_MODE_SHIFT = 1, AZP_MODE_XPLOR = 2 };
/* arithmetic of the pair / bond evaluation. FP32: FP32 arithmetic on exact
 * fixed-point displacements, compensated force / energy sums, FP64 cutoff
 * decision; state and integration stay FP64. */
enum azp_precision { AZP_FP64 = 0, AZP_FP32 = 1 };
enum azp_flow_kind { AZP_FLOW_CONSTANT = 0, AZP_FLOW_PARABOLIC = 1 };
enum azp_method { AZP_METHOD_LANGEVIN_FLOW = 0, AZP_METHOD_BROWNIAN_FLOW = 1 };

/* RNG stream identifiers, same values as src/RNGIdentifiers.h:20-27 */
#define AZP_RNG_DPD_GENERAL_WEIGHT 200u
#define AZP_RNG_BROWNIAN_FLOW 201u
#define AZP_RNG_LANGEVIN_FLOW 202u

/* ------------------------------------------------------------------ parameter structs
 * Field names, order and size of the reference param_type structs in HOOMD's
 * default double-precision build (HOOMD_LONGREAL_SIZE 64): sizeof is 32 bytes
 * (aligned(32)) for PerturbedLJ, ExpandedYukawa, Colloid, DPDGeneralWeight and
 * DoubleWell, 8 for Hertz (aligned(8)), 64 for Quartic, 16 for the ImageHarmonic
 * (HOOMD harmonic bond) record, 16 for the LJ93 wall and 32 for the Colloid wall
 * (src/PairEvaluatorPerturbedLennardJones.h:57-66, src/PairEvaluatorHertz.h:41-47,
 * src/BondEvaluatorDoubleWell.h:52-61, src/WallEvaluatorLJ93.h:50-58, ...).
 * Every table an entry point takes is an array of these records at that stride
 * (azp_record_size), indexed [type_i * ntypes + type_j] (pairs, symmetric),
 * [bond_type] (bonds) or [type] (walls): HOOMD's GPUArray<param_type> passes
 * straight through. A single-precision HOOMD build (Scalar = float) converts its
 * table with azp_params_from_single first. */
typedef struct { double sigma_6, epsilon_x_4, attraction_scale_factor, rwcasq; } azp_params_perturbed_lj;
typedef struct { double epsilon, kappa, delta, pad_; } azp_params_expanded_yukawa;
typedef struct { double epsilon; } azp_params_hertz;
typedef struct { double A, a_1, a_2, sigma_3; } azp_params_colloid;
typedef struct { double A, gamma, s, pad_; } azp_params_dpd_general_weight;
typedef struct { double k, r_0, b_1, b_2, U_0, sigma_6, epsilon_x_4, delta; } azp_params_quartic;
typedef struct { double r_1, r_diff, U_1, U_tilt; } azp_params_double_well;
typedef struct { double k, r_0; } azp_params_harmonic;

/* largest record, in doubles, of any pair / bond kind (buffer sizes) */
#define AZP_PAIR_PARAM_DOUBLES 4
#define AZP_BOND_PARAM_DOUBLES 8

/* record classes of azp_record_size / azp_params_from_single */
enum azp_record_class { AZP_RECORD_PAIR = 0, AZP_RECORD_BOND = 1, AZP_RECORD_WALL = 2 };
/* Bytes of one param_type record of (record class, kind): single == 0 gives the
 * double-precision layout every table argument uses, single != 0 the layout of a
 * HOOMD build with Scalar = float (aligned(16) / aligned(8) / aligned(4)
 * variants). Negative (AZP_ERR_INVALID) for an unknown class or kind. */
AZP_API int azp_record_size(int record_class, int kind, int single);
/* Widen n records of a single-precision HOOMD build (host memory, the layout
 * azp_record_size(cls, kind, 1) gives) into the double-precision layout the entry
 * points take (host memory, azp_record_size(cls, kind, 0) bytes each). */
AZP_API int azp_params_from_single(int record_class, int kind, const void* src, uint32_t n, double* dst);

/* Dict constructor / asDict of each param_type, host-only, no device work.
 * record: one record of azp_record_size(class, kind, 0) bytes.
 * values[] holds the Python parameter dict in this key order:
 *   PerturbedLennardJones: epsilon, sigma, attraction_scale_factor
 *   ExpandedYukawa:        epsilon, kappa, delta
 *   Hertz:                 epsilon
 *   Colloid:               A, a_1, a_2, sigma
 *   DPDGeneralWeight:      A, gamma, s
 *   Quartic:               k, r_0, b_1, b_2, U_0, sigma, epsilon, delta
 *   DoubleWell:            r_0, r_1, U_1, U_tilt
 *   ImageHarmonic:         k, r0
 * Replaces e.g. PairParametersPerturbedLennardJones(pybind11::dict) and asDict()
 * (src/PairEvaluatorPerturbedLennardJones.h:33-54). */
AZP_API int azp_pair_params_from_values(int kind, const double* values, double* record);
AZP_API int azp_pair_params_to_values(int kind, const double* record, double* values);
AZP_API int azp_bond_params_from_values(int kind, const double* values, double* record);
AZP_API int azp_bond_params_to_values(int kind, const double* record, double* values);
AZP_API int azp_pair_num_values(int kind);
AZP_API int azp_bond_num_values(int kind);

/* ------------------------------------------------------------------ system */
/* Orthorhombic periodic box centred on the origin: [-L/2, L/2) per axis. */
typedef struct { double L[3]; } azp_box;

/* Flow field passed by value (the reference passes the functor by value,
 * src/TwoStepLangevinFlowGPU.h:180). CONSTANT: u = (p0, p1, p2).
 * PARABOLIC: p0 = mean_velocity, p1 = separation; u_x = 1.5 p0 (1 - (y / (p1/2))^2). */
typedef struct { int32_t kind; int32_t pad_; double p[3]; } azp_flow;

/* Particle arrays, all DEVICE pointers, index order (not tag order):
 *   pos   [N][4] doubles: x, y, z, w; the low 32 bits of w's bit pattern hold the
 *         type (HOOMD's __int_as_scalar convention)
 *   vel   [N][4] doubles: vx, vy, vz, mass
 *   accel [N][3] doubles
 *   image [N][3] int32
 *   tag   [N] uint32 (RNG counter)
 *   diameter [N] doubles (only read when gamma comes from lambda * diameter) */
typedef struct {
    uint32_t N;
    uint32_t ntypes;
    double* pos;
    double* vel;
    double* accel;
    int32_t* image;
    const uint32_t* tag;
    const double* diameter;
    azp_box box;
} azp_system;

/* Force output. precision FP64: force [N][4] doubles (fx, fy, fz, energy),
 * virial [6][virial_pitch] doubles (xx, xy, xz, yy, yz, zz), may be NULL.
 * precision FP32: the same layouts in floats. Written, not accumulated, by the
 * pair driver; accumulated by the bond driver. */
typedef struct {
    void* force;
    void* virial;
    uint32_t virial_pitch;
    int32_t precision;
} azp_forces;

/* ------------------------------------------------------------------ device / library */
AZP_API int azp_abi_version(void);
/* number of visible CUDA devices (0 when none); never faults */
AZP_API int azp_device_count(void);
/* last CUDA error string of this thread's last failing call */
AZP_API const char* azp_last_error(void);

/* ------------------------------------------------------------------ neighbour list
 * Cell list binned at width >= max(r_cut + r_buff), full list (j listed for i and
 * i for j), pairs with r_cut == 0 never listed, exclusions removed. Membership is
 * decided in FP64 with the oracle's exact rounding (|dx|^2 < r_list^2), so the
 * sets are bit-exact. Layout: column-major neighbours[k * N + i], counts[i].
 * Replaces HOOMD's NeighborListGPUBinned behind hoomd.md.nlist.Cell(buffer=...).
 * N < 2^31 (AZP_ERR_INVALID otherwise; the same bound holds for azp_md_create). */
typedef struct azp_nlist azp_nlist;
AZP_API azp_nlist* azp_nlist_create(uint32_t N, uint32_t ntypes, uint32_t max_neighbors, int* status);
AZP_API void azp_nlist_destroy(azp_nlist* nl);
/* r_cut[ntypes*ntypes] (symmetric), host pointer */
AZP_API int azp_nlist_set_cutoffs(azp_nlist* nl, const double* r_cut, double r_buff);
/* exclusions as host CSR in index order: start[N+1], partners[] (both directions) */
AZP_API int azp_nlist_set_exclusions(azp_nlist* nl, const uint32_t* start, const uint32_t* partners);
/* unconditional rebuild at the current positions (synchronises the stream to
 * check overflow; grows and rebuilds on overflow) */
AZP_API int azp_nlist_build(azp_nlist* nl, const azp_system* sys, void* stream);
/* device views of the list, valid until the next build */
AZP_API int azp_nlist_view(const azp_nlist* nl, const uint32_t** counts, const uint32_t** neighbors,
                   uint32_t* max_neighbors, uint32_t* n_builds);
/* copy the list to HOST memory: counts[N], neighbors[max_neighbors * N]
 * (column-major); synchronises the stream */
AZP_API int azp_nlist_download(const azp_nlist* nl, uint32_t* counts, uint32_t* neighbors, void* stream);

/* ------------------------------------------------------------------ force drivers
 * Pair forces over the list (replaces gpu_compute_pair_forces<Eval>).
 * params: device table [ntypes*ntypes] of param_type records;
 * r_cut / r_on: device tables [ntypes*ntypes] (r_on may be NULL).
 * Overwrites out->force (and virial). Uses nl as its workspace (type-pair table,
 * FP32 fixed-point shadow): stream-ordered, no allocation, no synchronisation. */
AZP_API int azp_pair_forces(const azp_system* sys, azp_nlist* nl, int kind, const double* params,
                    const double* r_cut, const double* r_on, int shift_mode, const azp_forces* out,
                    void* stream);
/* threads per particle of azp_pair_forces: 1, 2, 4, 8, 16 or 32 */
AZP_API int azp_nlist_set_tpp(azp_nlist* nl, int tpp);

/* Pair forces without any allocation. No counterpart in the reference: it is
 * azp_pair_forces for callers that cannot allocate device memory (a host code
 * that reserves its whole device budget at start-up and lets plugins use only
 * buffers it owns, or a caller that cannot accept cudaMalloc's implicit device
 * synchronisation), so it cannot hold an azp_nlist workspace. The list comes in
 * as plain device arrays: counts[N] and neighbors[k * N + i] for
 * k < max_neighbors (the layout azp_nlist_view returns); everything else is as
 * for azp_pair_forces, with 4 threads per particle, so the results are the same.
 * Its scratch (type-pair table, FP32 position shadow) is one static device array
 * of this library, about 4.1 MB, held on every GPU that loads the library until
 * the process exits. Limits: N <= AZP_STATIC_MAX_N (else AZP_ERR_TOO_LARGE with a
 * message in azp_last_error) and ntypes <= 16 (else AZP_ERR_INVALID).
 * Preconditions, as for any caller-built list: every neighbors[k * N + i] with
 * k < min(counts[i], max_neighbors) is a particle index < N, and every type in
 * pos.w is < ntypes; the kernels read without range checks.
 * Every call looks the array's address up for the current device (with that
 * device current); the first call on a device may load the library's device code
 * there, so make that first call before any stream capture. Nothing is cached
 * between calls, so a device reset in between is harmless.
 * Calls share the array: two calls whose kernels overlap on the GPU (different
 * streams, or different host threads, on one device) race on it. Every call
 * rewrites what it reads, so nothing carries over from the previous call. */
#define AZP_STATIC_MAX_N 262144u
AZP_API int azp_pair_forces_static(const azp_system* sys, const uint32_t* counts, const uint32_t* neighbors,
                                   uint32_t max_neighbors, int kind, const double* params, const double* r_cut,
                                   const double* r_on, int shift_mode, const azp_forces* out, void* stream);

/* DPD with a general weight function (replaces HOOMD's gpu_compute_dpd_forces for
 * src/DPDPairEvaluatorGeneralWeight.h:165-255, instantiated in
 * src/PotentialPairDPDThermoGPUKernel.cu.inc:21-24): conservative, dissipative and
 * random pair forces over the list. params: device [ntypes^2] records (A, gamma, s,
 * -); r_cut: device [ntypes^2]; reads sys->pos, sys->vel (v, mass) and sys->tag.
 * The random draw of a pair comes from the stream (AZP_RNG_DPD_GENERAL_WEIGHT,
 * timestep, seed) at the ordered tag pair, so both particles see the same number.
 * Writes force and energy (conservative, half per particle) and the conservative
 * virial. Uses nl as its workspace; no allocation, no synchronisation. */
AZP_API int azp_dpd_forces(const azp_system* sys, azp_nlist* nl, const double* params, const double* r_cut,
                           double kT, double dt, uint64_t timestep, uint32_t seed, const azp_forces* out,
                           void* stream);

/* Moving harmonic barriers (replaces HarmonicBarrierGPU<Evaluator>::computeForces
 * and kernel::compute_harmonic_barrier, src/HarmonicBarrierGPU.cuh:50-83, with
 * src/PlanarBarrierEvaluator.h:36-56 and src/SphericalBarrierEvaluator.h:36-61).
 * geometry AZP_BARRIER_PLANAR: U = k/2 (y - H - offset)^2 above y = H + offset,
 * pushing -y; AZP_BARRIER_SPHERICAL: U = k/2 (r - R - offset)^2 beyond
 * r = R + offset, pushing inward. location: H or R, the value of the barrier's
 * variant at the timestep (HarmonicBarrier::makeEvaluator evaluates it, :121-130).
 * params: device [ntypes][2] doubles (k, offset). Each position is wrapped into
 * the box first (:168-170). OVERWRITES out->force (fx, fy, fz, energy) and zeroes
 * out->virial (may be NULL): the reference does not compute the virial (:177-179).
 * A location that fails the evaluator's valid(box) -- planar: -Ly/2 <= H < Ly/2;
 * spherical: R >= 0 and 2R <= each edge -- returns AZP_ERR_INVALID with
 * "Barrier position is invalid" in azp_last_error, before any device work.
 * FP64 output: FP64 arithmetic. FP32 output: FP32 arithmetic after the FP64
 * wrap and the cancelling difference (y - c, or r^2 - c^2). */
enum azp_barrier_geometry { AZP_BARRIER_PLANAR = 0, AZP_BARRIER_SPHERICAL = 1 };
AZP_API int azp_harmonic_barrier_forces(const azp_system* sys, int geometry, double location, const double* params,
                                        const azp_forces* out, void* stream);

/* Wall potentials (replaces gpu_compute_potential_external_forces<
 * EvaluatorWalls<WallEvaluator*>>, src/PotentialExternalWallGPUKernel.cu.inc:26-30,
 * with src/WallEvaluatorLJ93.h:100-133 and src/WallEvaluatorColloid.h:118-183;
 * walls as hoomd.wall.Sphere / Cylinder / Plane). For every wall the distance from
 * the particle to the wall surface is the argument of the energy-shifted
 * evaluator on the wall's active side (inside a sphere / cylinder with
 * inside != 0, outside otherwise; the normal's side of a plane; a particle on the
 * surface counts as active when open == 0). r_extrap > 0 continues the potential
 * linearly (constant force towards the active side) closer than r_extrap and on
 * the inactive side. Walls are visited spheres, cylinders, planes; cylinder axes
 * and plane normals need not be unit (they are normalised). A particle exactly at
 * a sphere's centre or on a cylinder's axis takes the surface point along a fixed
 * direction (+x; the first normal of the axis).
 * params: device [ntypes] records (azp_params_wall_*); r_cut, r_extrap: device
 * [ntypes]. OVERWRITES out->force (fx, fy, fz, energy) and out->virial
 * (F_a x_b, may be NULL). FP64 output: FP64 arithmetic. FP32 output: FP32
 * arithmetic except x - origin and R^2 - r^2 (FP64), so distances keep FP32
 * relative accuracy near a surface. */
enum azp_wall_kind { AZP_WALL_LJ93 = 0, AZP_WALL_COLLOID = 1 };
#define AZP_WALL_MAX_SPHERES 20
#define AZP_WALL_MAX_CYLINDERS 20
#define AZP_WALL_MAX_PLANES 60
typedef struct { double r; double origin[3]; int32_t inside; int32_t open; } azp_wall_sphere;
typedef struct { double r; double origin[3]; double axis[3]; int32_t inside; int32_t open; } azp_wall_cylinder;
typedef struct { double origin[3]; double normal[3]; int32_t open; int32_t pad_; } azp_wall_plane;
typedef struct {
    uint32_t n_spheres, n_cylinders, n_planes, pad_;
    const azp_wall_sphere* spheres;     /* host */
    const azp_wall_cylinder* cylinders; /* host */
    const azp_wall_plane* planes;       /* host */
} azp_walls;
/* param_type records (src/WallEvaluatorLJ93.h:31-58: 16 bytes, src/WallEvaluatorColloid.h:31-67: 32 bytes) */
typedef struct { double sigma_3, A; } azp_params_wall_lj93;
typedef struct { double c_1, c_2, a, pad_; } azp_params_wall_colloid;
/* dict constructor / asDict: values LJ93 {A, sigma}, Colloid {A, a, sigma} */
AZP_API int azp_wall_params_from_values(int kind, const double* values, double* record);
AZP_API int azp_wall_params_to_values(int kind, const double* record, double* values);
AZP_API int azp_wall_forces(const azp_system* sys, int kind, const azp_walls* walls, const double* params,
                            const double* r_cut, const double* r_extrap, const azp_forces* out, void* stream);

/* ------------------------------------------------------------------ velocity fields
 * Mass-averaged velocity per bin (replaces VelocityFieldComputeGPU<BinOp> with
 * src/VelocityFieldComputeGPU.cuh:35-72, src/CartesianBinningOperation.h and
 * src/CylindricalBinningOperation.h; the centre-of-mass velocity of
 * src/VelocityCompute.h is the Cartesian case with num_bins = {0, 0, 0}).
 * num_bins[d] = 0 ignores coordinate d; bins of coordinate d span
 * [lower[d], upper[d]) (Cartesian x, y, z; cylindrical r, theta in [0, 2 pi), z),
 * flattened with the last coordinate fastest. Each member's position is wrapped
 * into the box, its momentum m v turned into the bin's coordinates (cylindrical:
 * v_r, v_theta, v_z) and summed with its mass; velocity = momentum / mass, 0 in an
 * empty bin. Sums are exact 64-bit fixed-point integer sums of the contributions
 * rounded to 2^-40: the result does not depend on the order of the particles or
 * the schedule. A contribution of magnitude 2^22 or more sets AZP_EBIT_RANGE
 * (azp_vfield_error) and is left out. The object holds its accumulators; compute
 * is stream-ordered and allocates nothing. */
enum azp_binning_kind { AZP_BINNING_CARTESIAN = 0, AZP_BINNING_CYLINDRICAL = 1 };
typedef struct azp_vfield azp_vfield;
AZP_API azp_vfield* azp_vfield_create(int kind, const uint32_t* num_bins, const double* lower, const double* upper,
                                      int* status);
AZP_API void azp_vfield_destroy(azp_vfield* vf);
AZP_API uint32_t azp_vfield_num_bins(const azp_vfield* vf);
/* group: device index list of n_group members, or NULL for all sys->N particles
 * (reads sys->pos and sys->vel, mass in vel.w). Outputs are device arrays, each
 * may be NULL: mass [nbins], momentum [nbins][3], velocity [nbins][3]. */
AZP_API int azp_vfield_compute(azp_vfield* vf, const azp_system* sys, const uint32_t* group, uint32_t n_group,
                               double* mass, double* momentum, double* velocity, void* stream);
/* the accumulated error bits (AZP_EBIT_RANGE); synchronises the stream */
AZP_API int azp_vfield_error(azp_vfield* vf, uint32_t* err_word, void* stream);

/* Bond forces from a per-particle bond table (replaces
 * gpu_compute_bond_forces<Eval,2>): for particle i its bonds are
 * table[k * N + i] = (partner index, bond type) for k < n_bonds[i].
 * params: device table [nbondtypes] of param_type records. ACCUMULATES into out.
 * FP32 precision evaluates in FP32 on the FP64 minimum-image displacement.
 * AZP_BOND_IMAGE_HARMONIC (src/ImagePotentialBond.h:57-204) measures the
 * image-unwrapped displacement (x_i - x_j) + (img_i - img_j) L instead and needs
 * sys->image.
 * err: device uint32 error word (AZP_EBIT_BOND set when an evaluator refuses). */
AZP_API int azp_bond_forces(const azp_system* sys, const uint32_t* n_bonds, const uint32_t* table,
                    uint32_t table_height, int kind, const double* params, uint32_t nbondtypes,
                    const azp_forces* out, uint32_t* err, void* stream);

/* ------------------------------------------------------------------ adjoint (gradients)
 * Vector-Jacobian products of the force drivers, FP64. grad [N][4] holds dL/dF_i
 * (x, y, z) and dL/dU_i (w) for the per-particle forces and energies the forward
 * driver writes. Outputs: grad_pos [N][3] = dL/dx_i, and (optional) grad_params,
 * each particle's share of dL/d(param_type record fields) -- [N][4] for pairs,
 * [N][8] for bonds -- whose sum over particles is the parameter gradient (for
 * one type pair / bond type). All pair modes (r_on may be NULL). No counterpart
 * in the reference (azplugins has no gradients); they differentiate the drivers above. */
AZP_API int azp_pair_adjoint(const azp_system* sys, azp_nlist* nl, int kind, const double* params,
                             const double* r_cut, const double* r_on, int shift_mode, const double* grad,
                             double* grad_pos, double* grad_params, void* stream);
AZP_API int azp_bond_adjoint(const azp_system* sys, const uint32_t* n_bonds, const uint32_t* table, int kind,
                             const double* params, uint32_t nbondtypes, const double* grad, double* grad_pos,
                             double* grad_params, uint32_t* err, void* stream);

/* ------------------------------------------------------------------ integrator drivers
 * Particle subsets: group[n_group] index list, or NULL for all N particles.
 * gamma: device table [ntypes] (ignored when use_lambda != 0: gamma = lambda * diameter).
 * net_force: device [N][4] in the precision named by net_precision (FP64 doubles or FP32 floats). */
AZP_API int azp_langevin_step1(const azp_system* sys, const uint32_t* group, uint32_t n_group, double dt,
                       void* stream);
AZP_API int azp_langevin_step2(const azp_system* sys, const uint32_t* group, uint32_t n_group,
                       const void* net_force, int net_precision, const double* gamma, int use_lambda,
                       double lambda, azp_flow flow, double dt, double kT, uint64_t timestep,
                       uint32_t seed, int noiseless, void* stream);
AZP_API int azp_brownian_step(const azp_system* sys, const uint32_t* group, uint32_t n_group,
                      const void* net_force, int net_precision, const double* gamma, int use_lambda,
                      double lambda, azp_flow flow, double dt, double kT, uint64_t timestep,
                      uint32_t seed, int noiseless, double max_displacement, void* stream);

/* ------------------------------------------------------------------ RNG (test hook)
 * Three uniform doubles in (lo, hi) for (stream id, timestep, seed, tag), the same
 * numbers the integrators draw; computed on the device into out[3*n] for tags[n]. */
AZP_API int azp_uniform3(uint32_t rng_id, uint64_t timestep, uint32_t seed, const uint32_t* tags, uint32_t n,
                 double lo, double hi, double* out, void* stream);

/* ------------------------------------------------------------------ engine
 * Resident MD engine: particles kept in cell order in HBM, one fused
 * force + integrate kernel per step, conditional list rebuild and particle
 * re-sort on the device, steps replayed from captured CUDA graphs. Host-visible
 * state is always in tag order. */
typedef struct azp_md azp_md;

typedef struct {
    uint32_t N;
    uint32_t ntypes;
    azp_box box;
    int32_t precision;          /* azp_precision of the force evaluation */
    /* pair */
    int32_t pair_kind;          /* -1: no pair force */
    int32_t shift_mode;
    const double* pair_params;  /* host [ntypes*ntypes] param_type records */
    const double* r_cut;        /* host [ntypes*ntypes] */
    const double* r_on;         /* host [ntypes*ntypes] or NULL */
    double r_buff;
    /* bonds */
    int32_t bond_kind;          /* -1: no bond force */
    uint32_t nbondtypes;
    const double* bond_params;  /* host [nbondtypes] param_type records */
    uint32_t nbonds;
    const uint32_t* bonds;      /* host [nbonds][2] tags */
    const uint32_t* bond_types; /* host [nbonds] */
    int32_t exclude_bonds;      /* remove bonded pairs from the pair list */
    /* method */
    int32_t method;             /* azp_method */
    double dt;
    double kT;
    uint32_t seed;
    int32_t noiseless;
    const double* gamma;        /* host [ntypes] */
    int32_t use_lambda;
    double lambda;
    azp_flow flow;
    double max_displacement;    /* Brownian only; 0 = uncapped */
    double pair_force_cap;      /* > 0: |pair force| capped per pair (overlap relaxation); 0 = off */
    /* harmonic barrier added to the net force inside the fused step (the
     * reference's HarmonicBarrier in the integrator's forces, src/HarmonicBarrier.h) */
    int32_t barrier_geometry;   /* azp_barrier_geometry (read when barrier_params is set) */
    const double* barrier_params; /* host [ntypes][2] (k, offset); NULL: no barrier */
    /* wall potential added to the net force inside the fused step (the
     * reference's wall.LJ93 / wall.Colloid in the integrator's forces), with the
     * semantics of azp_wall_forces */
    int32_t wall_kind;          /* azp_wall_kind (read when walls is set) */
    const azp_walls* walls;     /* host; NULL: no walls */
    const double* wall_params;  /* host [ntypes] param_type records */
    const double* wall_r_cut;   /* host [ntypes] */
    const double* wall_r_extrap; /* host [ntypes] */
    /* pair_kind AZP_PAIR_DPD_GENERAL_WEIGHT: the thermostat temperature (the
     * dissipative and random terms, sqrt(6 kT gamma / dt)); needs the Langevin
     * method (with default gamma 0 and noiseless: HOOMD's ConstantVolume) */
    double dpd_kT;
    /* particles the method integrates, by type: bit t set means particles of type
     * t move (HOOMD's filter.Type group of the method, src/TwoStepLangevinFlow.h:35);
     * the others feel and exert forces but keep their positions and velocities.
     * 0 means every particle (filter.All). Types above 31 need 0. */
    uint32_t group_types;
} azp_md_config;

AZP_API azp_md* azp_md_create(const azp_md_config* cfg, int* status);
AZP_API void azp_md_destroy(azp_md* md);
/* Locations of the engine's harmonic barrier (its variant's values, host array):
 * location[r] belongs to timestep t_first + r, r < n <= AZP_MD_BARRIER_ROWS. The
 * forces of the positions at timestep t use the location of t: a Langevin step at
 * t evaluates t + 1 (HOOMD computes the net force of t + 1 between the two
 * halves), a Brownian step t; timesteps outside the rows take the nearest row, so
 * a constant barrier needs one row. Every location is checked as by
 * azp_harmonic_barrier_forces (AZP_ERR_INVALID, "Barrier position is invalid").
 * Must be called before the first run of an engine with a barrier; synchronises
 * the stream. */
#define AZP_MD_BARRIER_ROWS 65536u
AZP_API int azp_md_set_barrier_locations(azp_md* md, uint64_t t_first, uint32_t n, const double* location,
                                         void* stream);
/* Temperature of the method as a per-timestep table (HOOMD's Variant kT of
 * TwoStepLangevinFlow / TwoStepBrownianFlow, evaluated at the timestep of step
 * two or of the Brownian move, src/TwoStepLangevinFlow.h:194-219): kT[r] belongs
 * to timestep t_first + r, r < n <= AZP_MD_KT_ROWS; timesteps outside the rows
 * take the nearest row. Replaces azp_md_config.kT until the engine is destroyed;
 * the noise amplitudes sqrt(6 gamma kT / dt) are formed on the host with the
 * reference's operations. Synchronises the stream. */
#define AZP_MD_KT_ROWS 65536u
AZP_API int azp_md_set_temperatures(azp_md* md, uint64_t t_first, uint32_t n, const double* kT, void* stream);
/* Load state in TAG order from host (on_device == 0) or device pointers:
 * pos [N][4] (w = type as an integer-valued double), vel [N][4] (w = mass),
 * accel [N][3], image [N][3], diameter [N] or NULL. */
AZP_API int azp_md_set_state(azp_md* md, const double* pos, const double* vel, const double* accel,
                     const int32_t* image, const double* diameter, uint64_t timestep, int on_device,
                     void* stream);
AZP_API int azp_md_get_state(azp_md* md, double* pos, double* vel, double* accel, int32_t* image,
                     uint64_t* timestep, int on_device, void* stream);
/* Advance `steps` timesteps (HOOMD order: step one, forces, step two).
 * Enqueues only: errors (list overflow, refused bond, non-finite position) are
 * read with azp_md_error. */
AZP_API int azp_md_run(azp_md* md, uint64_t steps, void* stream);
/* azp_md_run, then synchronise and check: on a list overflow the state saved at
 * entry is restored, the list grown to the largest count seen, and the steps run
 * again (HOOMD likewise grows its list and recomputes). */
AZP_API int azp_md_run_checked(azp_md* md, uint64_t steps, void* stream);
/* Net force [N][4] (fx, fy, fz, energy) and virial [N][6] at the current
 * positions, in tag order, FP64 (host or device pointers). */
AZP_API int azp_md_forces(azp_md* md, double* force, double* virial, int on_device, void* stream);
/* Global sums in FP64: out[0] potential energy, out[1] kinetic energy,
 * out[2..7] virial xx, xy, xz, yy, yz, zz, out[8] list builds so far (host out). */
AZP_API int azp_md_thermo(azp_md* md, double* out, void* stream);
/* The accumulated device error word (AZP_EBIT_*), 0 when clean. */
AZP_API int azp_md_error(azp_md* md, uint32_t* err_word, void* stream);
/* number of kernel launches issued by the last azp_md_run */
AZP_API uint64_t azp_md_last_launches(const azp_md* md);
/* Measurement hook: launch the fused step kernel alone `reps` times (no list
 * checks or rebuilds; the state advances and is only fit for timing afterwards)
 * between two CUDA events on `stream`; *ms = mean milliseconds per launch. */
AZP_API int azp_md_time_step_kernel(azp_md* md, int reps, float* ms, void* stream);

/* ------------------------------------------------------------------ batched replicas
 * Many independent systems (own box, pair parameters, seed; one particle type
 * each) advanced together: one fused force + Langevin launch per timestep for
 * all of them, replayed from a CUDA graph, list rebuilds as a graph conditional.
 * Host arrays are packed replica after replica (replica r at offset
 * sum_{q<r} N_q, in tag order within the replica). No counterpart in the
 * reference, which advances one system per HOOMD simulation. */
typedef struct azp_batch azp_batch;
typedef struct {
    uint32_t nsys;
    const uint32_t* N;          /* host [nsys] */
    const double* L;            /* host [nsys][3] */
    int32_t precision;
    int32_t pair_kind;
    int32_t shift_mode;
    const double* pair_params;  /* host [nsys] param_type records */
    const double* r_cut;        /* host [nsys] */
    double r_buff;
    double dt, kT, gamma;
    const uint32_t* seeds;      /* host [nsys] */
    int32_t noiseless;
    int32_t pad_;
    azp_flow flow;
} azp_batch_config;
AZP_API azp_batch* azp_batch_create(const azp_batch_config* cfg, int* status);
AZP_API void azp_batch_destroy(azp_batch* b);
/* pos [sumN][4] (w ignored), vel [sumN][4] (w = mass), accel [sumN][3] or NULL,
 * image [sumN][3] or NULL; host pointers */
AZP_API int azp_batch_set_state(azp_batch* b, const double* pos, const double* vel, const double* accel,
                                const int32_t* image, uint64_t timestep, void* stream);
AZP_API int azp_batch_get_state(azp_batch* b, double* pos, double* vel, double* accel, int32_t* image,
                                void* stream);
AZP_API int azp_batch_run(azp_batch* b, uint64_t steps, void* stream);
AZP_API int azp_batch_error(azp_batch* b, uint32_t* err_word, uint32_t* n_builds, void* stream);
/* threads per particle of the fused step (the autotuner's first knob) */
AZP_API int azp_batch_set_tpp(azp_batch* b, int tpp);
/* threads per block of the fused step: 64, 128, 256 (default) or 512 (the
 * autotuner's second knob) */
AZP_API int azp_batch_set_block(azp_batch* b, int block);
AZP_API uint64_t azp_batch_last_launches(const azp_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* AZPLUGINS_GB300_H_ */
