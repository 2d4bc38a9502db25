/* svxg_types.h - plain C graph, material and option records of the GB300 stress solve.
 *
 * These are the C-ABI images of the reference's C++ inputs:
 *   svxg_node     <- svx::SNode            core/include/svx/stress/stress.hpp:21-26
 *   svxg_bond     <- svx::SBond            core/include/svx/stress/stress.hpp:28-51
 *   svxg_material <- svx::Material (the fields the solve reads)
 *                                          core/include/svx/material/material.hpp:47-57
 *   svxg_amg_options    <- svx::AmgOptions core/include/svx/solve/amg.hpp:46-69
 *   svxg_stress_options <- svx::StressOptions core/include/svx/stress/stress.hpp:68-72
 *   svxg_pcg_result     <- svx::PcgResult  core/include/svx/solve/amg.hpp:120-125
 *
 * Layouts are fixed (no padding left to the compiler) so that ctypes, cgo or a C++ host can
 * fill them directly. Vectors are 3 doubles. Booleans are one byte.
 */
#ifndef SVXG_TYPES_H
#define SVXG_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct svxg_v3 {
  double x, y, z;
} svxg_v3;

/* A fragment: 6 DOFs (translation, rotation about c). 40 bytes. */
typedef struct svxg_node {
  svxg_v3 c;       /* centre (the solve's frame), m */
  double mass;     /* kg */
  uint8_t fixed;   /* pinned: no DOFs */
  uint8_t gone;    /* retired: an identity row, no bonds */
  uint8_t pad[6];
} svxg_node;

/* An interface between two fragments (b < 0: a fixed support). 216 bytes. */
typedef struct svxg_bond {
  int32_t a, b;
  uint8_t broken;     /* severed */
  uint8_t in_k;       /* its stiffness is in the assembled K (kept by the problem) */
  uint8_t ma, mb;     /* material ids (0..126) */
  uint8_t sectioned;  /* section strengths below, else the weaker material's */
  uint8_t pad[3];
  svxg_v3 n, t1, t2;  /* local frame: n from a towards b */
  double area;        /* m^2 */
  svxg_v3 p;          /* section centroid */
  double s1, s2;      /* second moments of area about p along t1, t2 */
  double c1, c2;      /* extreme fibre distances */
  double rmax;        /* largest distance of the section from p */
  double la, lb;      /* lengths of the two sides along n */
  double strength;    /* design strength multiplier */
  float ft, fb, fc, coh, mu; /* section strengths (Pa) and friction */
  int32_t faces;
  int32_t tag;
  int32_t pad2;
} svxg_bond;

#define SVXG_MAX_MATERIALS 127

/* What the solve reads of a material. 64 bytes. A table always holds SVXG_MAX_MATERIALS
 * resolved entries (ids never registered carry id 0's properties, as the reference table's
 * lookup returns). */
typedef struct svxg_material {
  double E, G, rho;
  double ft, fb, fc, cohesion, friction;
} svxg_material;

/* A moving piece's rigid-body state for its loads (the world's Body, core/include/svx/phys/rigid.hpp):
 * centre of mass x (world), orientation q (x, y, z, w), centre of mass in the shape frame com,
 * angular velocity w (world), inertia and its inverse (body frame, row-major), 1 / mass, and
 * gravity's magnitude (along -z). 200 bytes. */
typedef struct svxg_body_state {
  svxg_v3 x;
  double q[4];
  svxg_v3 com;
  svxg_v3 w;
  double inertia[9];
  double inv_inertia[9];
  double inv_mass;
  double gravity;
} svxg_body_state;

/* A point force on a piece: F at point p (both world), acting on graph node `node` (the world's
 * fragment-to-node map; out of range: it enters the piece's motion only). 56 bytes. */
typedef struct svxg_point_force {
  svxg_v3 F;
  svxg_v3 p;
  int32_t node;
  int32_t pad;
} svxg_point_force;

typedef struct svxg_amg_options {
  int32_t coarse_max;     /* dense solve at or below this many nodes (48) */
  int32_t smoothed;       /* smoothed aggregation (1) */
  double strength;        /* strength-of-connection threshold (0.1) */
  double coarse_scale;    /* unsmoothed coarse operator scale (0.6) */
  int32_t max_levels;     /* 16 */
  int32_t gamma;          /* 1: V-cycle (the only cycle the reference runs) */
  int32_t sgs;            /* reference smoother switch (1); recorded for the work counters */
  int32_t sweeps;         /* smoother sweeps per side (1) */
  int32_t cheb_degree;    /* 3 */
  int32_t dense_work_per_unknown; /* 0 */
  int32_t coarsen_dense;  /* 1 */
  int32_t reaggregate;    /* 1 */
} svxg_amg_options;

/* Arithmetic of the solve. */
enum {
  SVXG_PRECISION_FP64 = 0,      /* FP64 K, FP64 PCG; FP32 V-cycle (as the reference) */
  SVXG_PRECISION_MIXED = 1,     /* the mixed-precision policy: FP32 V-cycle, the multigrid built
                                   with FMAs and a tree-summed power-iteration norm (values within
                                   rounding of the reference's), FP64 K and Krylov vectors; the
                                   solve states its error against the FP64 solution */
  SVXG_PRECISION_MIXED_ALL = 2  /* that, and FP32 K and Krylov vectors inside FP64 iterative
                                   refinement (inner sequences) */
};

typedef struct svxg_stress_options {
  double rtol;             /* 2e-3 */
  svxg_amg_options amg;
  int32_t amg_min_nodes;   /* 160: smaller graphs get block-Jacobi */
  int32_t precision;       /* SVXG_PRECISION_* */
} svxg_stress_options;

typedef struct svxg_pcg_result {
  int32_t iters;
  int32_t converged;
  int32_t breakdown;
  int32_t pad;
  double rel_res;
} svxg_pcg_result;

/* Bond loads in bond terms (reference BondLoad, core/include/svx/stress/stress.hpp:61-63). */
typedef struct svxg_bond_load {
  double N, V1, V2, T, M1, M2;
} svxg_bond_load;

enum { SVXG_FAIL_NONE = 0, SVXG_FAIL_TENSION = 1, SVXG_FAIL_CRUSH = 2, SVXG_FAIL_SHEAR = 3 };

/* A bond's interface before it is a bond: the world's accumulator of the voxel faces two
 * fragments share (all axes), or of one fragment's faces on a support along one axis, and of the
 * junction samples where it meets another grid (SecHead / SecAcc,
 * core/src/world/world_internal.hpp:106-128). Its faces are faces[first_face .. + faces), its
 * junction samples junctions[first_junction .. + junctions). 64 bytes. */
typedef struct svxg_section {
  int32_t a, b;          /* nodes; b < 0: a support */
  int64_t first_face;
  int32_t faces;
  uint8_t axis;          /* a support's face axis (0..2) */
  int8_t sign;           /* a support's side of a: the normal from a to the support is sign e_axis */
  uint8_t ma, mb;        /* materials of the two sides (a support's: its own) */
  uint8_t sectioned;     /* 1: strengths from the faces' voxels (section_strengths) */
  uint8_t pad;
  uint16_t grid;         /* the lattice of its faces (index into the lattice table; 0 without one) */
  int32_t junctions;
  int64_t first_junction;
  double h;              /* voxel size of the faces' lattice (m) */
  double strength_a, strength_b;  /* the two sides' strength multipliers */
} svxg_section;

/* One voxel face of an interface: the face between voxel (x, y, z) of the lattice and its
 * +axis neighbour; sign +1 when a is on the lower side. The two voxels as the world stores them
 * (core/include/svx/world/grid.hpp:27-38: 0 air, else material id + 1 in the low 7 bits) and
 * their damage (0 intact .. 255 no strength left). 20 bytes. */
typedef struct svxg_face {
  int32_t x, y, z;
  uint8_t axis;
  int8_t sign;
  uint8_t vox_lo, vox_hi;
  uint8_t damage_lo, damage_hi;
  uint8_t pad[2];
} svxg_face;

/* A lattice in the frame the bonds are made in (LatticeXf, core/include/svx/phys/rigid.hpp:85-95):
 * x_frame = off + R x_lattice unless identity. 112 bytes. */
typedef struct svxg_lattice {
  double off[3];
  double R[9];           /* row-major */
  double h;              /* its voxel size (m) */
  uint8_t identity;
  uint8_t pad[7];
} svxg_lattice;

/* A junction sample (JSample, world_internal.hpp:71-79): sample `sub` of face `face` (axis x 2
 * + 1 for the +axis face) of voxel v of lattice vg lands in voxel o of lattice og (kind 1: in
 * the unknown world - it holds what reaches into it); sign +1 when the face normal points from a
 * towards b (or out of a, to a support); weight its share of the face (the samples of both sides
 * count half each). The two voxels and their damage as the faces'. 40 bytes. */
typedef struct svxg_junction {
  int32_t v[3], o[3];
  uint16_t vg, og;
  uint8_t face, sub, kind;
  int8_t sign;
  float weight;
  uint8_t vox_v, vox_o, damage_v, damage_o;
} svxg_junction;

/* The judge's break rounds of one structure: World::Impl::judge (core/src/world/world.cpp:1162-1277)
 * with the solve restarts of World::Impl's tick (world.cpp:1041-1110) and detach_unsupported
 * (world.cpp:1371-1458, graph_components world_internal.hpp:660-705). Defaults: WorldConfig and
 * WorldParams (core/include/svx/world/world.hpp:116, :140-153). */
typedef struct svxg_cascade_options {
  double rtol;                  /* stress_rtol, 3e-3 */
  double fragility;             /* 1 */
  double dif;                   /* dynamic increase factor of a sudden load change, 1.5 */
  double break_band;            /* a round breaks phi >= max(1, band x max phi), 0.85 */
  int32_t max_breaks_per_round; /* 256 (at most 65536 here) */
  int32_t max_rounds;           /* 400 */
  int32_t maxit;                /* iterations of a solve before it restarts, 120 (world.cpp:1074) */
  int32_t solve_restarts;       /* unconverged restarts in a row before the structure is left, 60 */
  int32_t rebuild_after;        /* a converged solve longer than this rebuilds a stale
                                   preconditioner before the next one, 60 (world.cpp:1109) */
  int32_t shock;                /* 1: the first judgement blends from the judged loads (a sudden
                                   load change), as every judgement after a round of breaks does */
  int32_t detach;               /* 1: after a round, parts no longer held by a support retire */
  int32_t pad;
} svxg_cascade_options;

enum {
  SVXG_CASCADE_SETTLED = 0,    /* a judgement found no bond at or over its strength */
  SVXG_CASCADE_MAX_ROUNDS = 1, /* max_rounds rounds broke bonds, and some are still over */
  SVXG_CASCADE_ABANDONED = 2,  /* solve_restarts restarts in a row did not converge */
  SVXG_CASCADE_BREAKDOWN = 3,  /* a solve broke down (not positive definite, or non-finite) */
  SVXG_CASCADE_SINGULAR = 4    /* assemble() found a singular diagonal */
};

typedef struct svxg_cascade_result {
  int32_t status;         /* SVXG_CASCADE_* */
  int32_t rounds;         /* rounds that broke bonds */
  int32_t bonds_broken;   /* by the rounds (bonds of retired nodes not counted) */
  int32_t nodes_retired;
  int32_t solves;
  int32_t restarts;       /* unconverged solves restarted, in all */
  int64_t pcg_iters;
  double max_utilization; /* of the last judgement */
  double rel_res;         /* of the last solve */
} svxg_cascade_result;

/* A loose piece's break rounds within one substep: World::Impl::body_stress_run's rounds
 * (core/src/world/world_pieces.cpp:614-808) on its load (inertial relief and point forces, built
 * by the caller). Defaults: WorldConfig (core/include/svx/world/world.hpp:150, :165-176, :269). */
typedef struct svxg_piece_options {
  double rtol;                  /* body_stress_rtol, 1e-2 */
  double fragility;             /* 1 */
  double break_band;            /* 0.85 */
  double round_fraction;        /* impact_round_fraction: a round breaks at least this fraction
                                   of the bonds over strength, 0.25 */
  double energy;                /* what the impact dissipates (J); < 0: a resting load, no limit */
  double fracture_energy;       /* x the materials' fracture energies, 1 */
  double crush_energy;          /* crushing a bond costs this x its fracture energy, 20 */
  double chip_fraction;         /* parts lighter than this x the piece are chips, 0.04 */
  int32_t maxit;                /* body_stress_maxit, 60 */
  int32_t rounds;               /* impact_rounds, 8 */
  int32_t max_breaks_per_round; /* 256 */
  int32_t pad;
} svxg_piece_options;

enum {
  SVXG_PIECE_SETTLED = 0,      /* a round found no bond at or over its strength */
  SVXG_PIECE_ENERGY = 1,       /* the impact's energy could not pay for the next crack */
  SVXG_PIECE_APART = 2,        /* the piece came apart (a part heavier than a chip) */
  SVXG_PIECE_LAST_ROUND = 3,   /* the last round broke bonds */
  SVXG_PIECE_SOLVE_FAILED = 4, /* a solve did not converge even on a rebuilt preconditioner */
  SVXG_PIECE_NO_PIN = 5,       /* bonds broke but the piece has no pinned node to split from */
  SVXG_PIECE_SINGULAR = 6      /* assemble() found a singular diagonal */
};

typedef struct svxg_piece_result {
  int32_t status;          /* SVXG_PIECE_* */
  int32_t checks;          /* rounds solved and judged */
  int32_t bonds_broken;
  int32_t chips;           /* chip nodes retired (their loads moved to the piece) */
  int32_t pcg_iters;
  int32_t rebuilt;         /* the preconditioner was rebuilt once */
  double spent;            /* fracture energy paid */
  double first_max_utilization;  /* the first round's largest phi (the body's last_phi) */
  double max_utilization;  /* the last round's */
} svxg_piece_result;

static inline svxg_piece_options svxg_default_piece_options(void) {
  svxg_piece_options o;
  o.rtol = 1e-2;
  o.fragility = 1.0;
  o.break_band = 0.85;
  o.round_fraction = 0.25;
  o.energy = -1.0;
  o.fracture_energy = 1.0;
  o.crush_energy = 20.0;
  o.chip_fraction = 0.04;
  o.maxit = 60;
  o.rounds = 8;
  o.max_breaks_per_round = 256;
  o.pad = 0;
  return o;
}

static inline svxg_cascade_options svxg_default_cascade_options(void) {
  svxg_cascade_options o;
  o.rtol = 3e-3;
  o.fragility = 1.0;
  o.dif = 1.5;
  o.break_band = 0.85;
  o.max_breaks_per_round = 256;
  o.max_rounds = 400;
  o.maxit = 120;
  o.solve_restarts = 60;
  o.rebuild_after = 60;
  o.shock = 0;
  o.detach = 1;
  o.pad = 0;
  return o;
}

/* Defaults of the reference's option records. */
static inline svxg_stress_options svxg_default_options(void) {
  svxg_stress_options o;
  o.rtol = 2e-3;
  o.amg.coarse_max = 48;
  o.amg.smoothed = 1;
  o.amg.strength = 0.1;
  o.amg.coarse_scale = 0.6;
  o.amg.max_levels = 16;
  o.amg.gamma = 1;
  o.amg.sgs = 1;
  o.amg.sweeps = 1;
  o.amg.cheb_degree = 3;
  o.amg.dense_work_per_unknown = 0;
  o.amg.coarsen_dense = 1;
  o.amg.reaggregate = 1;
  o.amg_min_nodes = 160;
  o.precision = SVXG_PRECISION_FP64;
  return o;
}

#ifdef __cplusplus
}
#endif

#endif /* SVXG_TYPES_H */
