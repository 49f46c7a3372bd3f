/*
 * lbm_gb300.h — C ABI of the GB300 (sm_103a) D2Q9 lattice-Boltzmann step.
 *
 * This is the boundary the Python drop-in (package taichi_lbm) binds through
 * ctypes.  taichi-lbm itself has no FFI: every per-step operation is a Taichi
 * @ti.kernel method.  Each entry point below replaces one of those methods and
 * names it (file:line inside the taichi-lbm project).
 *
 * Conventions
 *  - Every call returns int: LBM_OK (0) or a negative LBM_ERR_*; the message
 *    of the last failure on the calling thread is read with lbm_last_error().
 *    No C++ exception crosses this boundary.
 *  - All buffers are DEVICE pointers owned by the caller (PyTorch allocates
 *    and frees them); the library never frees caller memory.
 *  - Work is enqueued on the given CUDA stream (cudaStream_t passed as
 *    void*; NULL = legacy default stream) and is stream-ordered: calls on one
 *    stream run in call order, nothing here synchronizes the host.
 *  - A plan (LbmPlan) is used by one host thread at a time.
 *
 * Lattice layout (structure of arrays, x fastest, rows padded):
 *  node (i, j) of a scalar field is at  j*pitch + i,  0 <= i < nx, 0 <= j < ny
 *  population k of node (i, j) is at    k*ny*pitch + j*pitch + i
 *  vector component c is at             c*ny*pitch + j*pitch + i
 *  psi (one-node halo) of node (i, j) at (j+1)*psi_pitch + (i+1), -1 <= i <= nx,
 *  -1 <= j <= ny.  pitch and psi_pitch are multiples of 32 elements and the
 *  base pointers are 128-byte aligned.
 *  Velocity set (c_k) and weights follow taichi_lbm/lbm.py:44-45:
 *  k: 0 (0,0) 1 (1,0) 2 (0,1) 3 (-1,0) 4 (0,-1) 5 (1,1) 6 (-1,1) 7 (-1,-1) 8 (1,-1)
 *
 *  Groups are the reference's MaskAndGroup node lists
 *  (taichi_lbm/BoundaryCondition.py:8-12): int32 pairs (i, j), n entries.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_GB300_ABI_VERSION 4

enum {
  LBM_OK = 0,
  LBM_ERR_ARG = -1,         /* invalid argument or size */
  LBM_ERR_CUDA = -2,        /* a CUDA runtime call failed */
  LBM_ERR_UNSUPPORTED = -3, /* combination this build does not run */
  LBM_ERR_STATE = -4        /* call out of order (e.g. plan not bound) */
};

/* collision models (taichi_lbm/CollisionEngine.py) */
enum { LBM_BGK = 0, LBM_TRT = 1, LBM_MRT = 2 };
/* fluid models (taichi_lbm/FluidModels.py) */
enum { LBM_NEWTONIAN = 0, LBM_POWERLAW = 1 };
/* population storage for the fused path: fp32; fp16 / bf16 shifted; int16
 * fixed point shifted (steps of 2^-19, |f_k - w_k rho_ref| < 1/16, every
 * collision conserves each node's stored mass exactly; direct and prefetch
 * pipelines, not Shan-Chen) */
enum { LBM_STORE_F32 = 0, LBM_STORE_F16S = 1, LBM_STORE_BF16S = 2, LBM_STORE_I16S = 3 };
/* pseudopotentials (taichi_lbm/EOS.py) */
enum { LBM_EOS_SC = 0, LBM_EOS_VDW = 1, LBM_EOS_RK = 2, LBM_EOS_PR = 3, LBM_EOS_CS = 4 };
/* boundary-condition kinds (taichi_lbm/BoundaryCondition.py) */
enum {
  LBM_BC_FLUID = 0,         /* FluidBoundary, BoundaryCondition.py:452-455 (no-op)     */
  LBM_BC_VELOCITY_BB = 1,   /* VelocityBB, BoundaryCondition.py:80-102                  */
  LBM_BC_VELOCITY_EQ = 2,   /* VelocityEquilibrium, BoundaryCondition.py:132-147        */
  LBM_BC_VELOCITY_NEEM = 3, /* VelocityNEEM, BoundaryCondition.py:149-166               */
  LBM_BC_PRESSURE_ABC = 4,  /* PressureABC, BoundaryCondition.py:177-205                */
  LBM_BC_PRESSURE_NEEM = 5, /* PressureNEEM, BoundaryCondition.py:209-226               */
  LBM_BC_OPEN_NEUMANN = 6,  /* OpenNeumann, BoundaryCondition.py:315-334                */
  LBM_BC_OPEN_CONV1 = 7,    /* OpenConvective1order, BoundaryCondition.py:337-359       */
  LBM_BC_OPEN_CONV2 = 8,    /* OpenConvective2order, BoundaryCondition.py:362-390       */
  LBM_BC_OPEN_EXTRAP = 9,   /* OpenExtrapolation, BoundaryCondition.py:394-411          */
  LBM_BC_PERIODIC = 10,     /* PeriodicAllBoundary, BoundaryCondition.py:419-432        */
  LBM_BC_INSIDE = 11,       /* InsideBoundary, BoundaryCondition.py:435-449             */
  LBM_BC_BOUNCEBACK = 12    /* BounceBackWall, BoundaryCondition.py:231-259             */
};

/* Lattice fields — the device-side LBField (taichi_lbm/lbm.py:5-56), single
 * component.  Unused pointers may be NULL for calls that do not touch them. */
typedef struct LbmLattice {
  int32_t nx, ny;
  int32_t pitch;      /* elements per row of every [ny][pitch] plane        */
  int32_t psi_pitch;  /* elements per row of psi (ny+2 rows)               */
  float* f;           /* [9][ny][pitch] populations (post-stream)          */
  float* f2;          /* [9][ny][pitch] populations (post-collision)       */
  float* rho;         /* [ny][pitch]                                        */
  float* total_rho;
  float* pressure;
  float* total_pressure;
  float* shear_rate;
  float* temperature; /* LBField.T                                          */
  float* vel;         /* [2][ny][pitch]                                     */
  float* body_force;
  float* sc_force;    /* LBField.SCforce                                    */
  float* psi;         /* ShanChenModel.psi_field, one-node halo             */
  int32_t* mask;      /* [ny][pitch] 1 fluid, -1 solid                      */
  uint16_t* links;    /* [ny][pitch] LBField.neighbor in bit form: bit k set
                         = link k has a source (neighbor != -1); bit 15 set =
                         node was classified (non-solid at classify time)   */
  float gravity[2];   /* LBField.gravity_force                              */
} LbmLattice;

/* Immersed-boundary nodes (taichi_lbm/ibm.py:7-14, the IBMNodes fields),
 * n nodes as [n][2] float arrays in device memory. */
typedef struct LbmIBNodes {
  int64_t n;
  float* pos;
  float* vel;
  float* vel_desired;
  float* force;
  float* force_temp;
} LbmIBNodes;

/* Collision operator state (taichi_lbm/CollisionEngine.py:6-451). */
typedef struct LbmCollision {
  int32_t model;        /* LBM_BGK / LBM_TRT / LBM_MRT                           */
  int32_t fluid_model;  /* LBM_NEWTONIAN / LBM_POWERLAW                          */
  float nu;             /* shearviscosity[0] (and NewtonianFluid.nu)              */
  float nu_bulk;        /* bulkviscosity[0] (MRT)                                 */
  float magic;          /* magic[0] (TRT)                                         */
  float tau_min, tau_max;  /* Collision.tau_min / tau_max (CollisionEngine.py:10-11) */
  float pl_m, pl_n;     /* PowerLawFluid.m / .n (FluidModels.py:20-29)            */
  float* tau;           /* BGK   [ny][pitch]                                      */
  float* tau_sym;       /* TRT   [ny][pitch]                                      */
  float* tau_antisym;   /* TRT   [ny][pitch]                                      */
  float* diag;          /* MRT   [9][ny][pitch]                                   */
  float m_inverse[81];  /* MRT   MRTCollision.M_inverse, row-major                */
} LbmCollision;

/* Pseudopotential parameters (taichi_lbm/EOS.py:5-95). */
typedef struct LbmEos {
  int32_t kind;         /* LBM_EOS_*                                              */
  float a, b, R, G;     /* Pseudopotential a, b, R, G                             */
  float rho0;           /* SC_psi rho0                                            */
  float omega;          /* PR_psi omega                                           */
  float T_cr;           /* temperature_cr                                         */
} LbmEos;

/* One boundary condition (taichi_lbm/BoundaryCondition.py:57-226, 264-449). */
typedef struct LbmBoundary {
  int32_t kind;         /* LBM_BC_*                                               */
  int32_t direction;    /* PlaneBoundary.direction (1..4)                         */
  float rho_value;      /* PressureBoundary.rho_value                             */
  float velocity[2];    /* VelocityBoundary.velocity_value                        */
  const float* velocity_per_node; /* n x 2 per-node values (group order) or NULL:
                                     the BoundarySpec.value_fn extension        */
  float g_coh;          /* OpenConvective2order: ShanChenForceC1.g_coh            */
  LbmEos eos;           /* OpenConvective2order: the psi model                    */
} LbmBoundary;

/* ---------------------------------------------------------------- library */
int lbm_abi_version(void);
/* Copy the calling thread's last error message into buf (always terminated). */
int lbm_last_error(char* buf, int64_t buflen);

/* ------------------------------------------------------- per-stage kernels
 * One launch each, over the given group, exactly the reference method's
 * effect on the fields.                                                      */

/* LBField.neighbor_classify — taichi_lbm/lbm.py:127-142 */
int lbm_neighbor_classify(const LbmLattice* lat, void* stream);
/* LBField.init_LBM — taichi_lbm/lbm.py:119-125 (f = f2 = feq(rho, vel)) */
int lbm_init_feq(const LbmLattice* lat, const int32_t* group, int64_t n, void* stream);
/* MacroscopicEngine.density — taichi_lbm/lbm.py:153-164 */
int lbm_density(const LbmLattice* lat, const int32_t* group, int64_t n, void* stream);
/* MacroscopicEngine.pressure0 / pressure1 — taichi_lbm/lbm.py:166-182 */
int lbm_pressure(const LbmLattice* lat, const int32_t* group, int64_t n, int32_t with_sc,
                 float g_coh, void* stream);
/* MacroscopicEngine.force_density — taichi_lbm/lbm.py:215-220 */
int lbm_force_density(const LbmLattice* lat, const int32_t* group, int64_t n, void* stream);
/* MacroscopicEngine.velocity — taichi_lbm/lbm.py:223-237 */
int lbm_velocity(const LbmLattice* lat, const int32_t* group, int64_t n, void* stream);

/* IBEngine.InterpolateBodyVelocities — taichi_lbm/ibm.py:201-223: each node's
 * velocity from the lattice velocity on its floor..ceil stencil, and its
 * correction force 2 (vel_desired - vel) into force_temp, added to force. */
int lbm_ibm_interpolate(const LbmLattice* lat, const LbmIBNodes* nodes, void* stream);
/* IBEngine.SpreadBodyForces — taichi_lbm/ibm.py:225-246: each node's
 * force_temp spread on its stencil into the lattice velocity (/ 2 total_rho)
 * and body force (x rho / total_rho).  Adds are atomic. */
int lbm_ibm_spread(const LbmLattice* lat, const LbmIBNodes* nodes, void* stream);

/* {BGK,TRT,MRT}Collision.initTau — CollisionEngine.py:65-70, 149-155, 301-318 */
int lbm_collision_init_tau(const LbmLattice* lat, const LbmCollision* c, const int32_t* group,
                           int64_t n, void* stream);
/* {BGK,TRT,MRT}Collision.shear_rate — CollisionEngine.py:80-92, 166-178, 332-377 */
int lbm_collision_shear_rate(const LbmLattice* lat, const LbmCollision* c, const int32_t* group,
                             int64_t n, void* stream);
/* {BGK,TRT,MRT}Collision.relaxation_time — CollisionEngine.py:72-78, 157-164, 322-329 */
int lbm_collision_relaxation_time(const LbmLattice* lat, const LbmCollision* c,
                                  const int32_t* group, int64_t n, void* stream);
/* {BGK,TRT,MRT}Collision.apply — CollisionEngine.py:96-110, 223-245, 424-451 */
int lbm_collision_apply(const LbmLattice* lat, const LbmCollision* c, const int32_t* group,
                        int64_t n, void* stream);

/* ShanChenForceC1.update_psi — taichi_lbm/ExternalForce.py:42-47 */
int lbm_sc_update_psi(const LbmLattice* lat, const LbmEos* eos, const int32_t* group, int64_t n,
                      void* stream);
/* ShanChenForceC1.cau_SCforce — taichi_lbm/ExternalForce.py:50-63 */
int lbm_sc_force(const LbmLattice* lat, float g_coh, const int32_t* group, int64_t n, void* stream);
/* PeriodicPsi_LR (axis 0) / PeriodicPsi_BT (axis 1) — SCBoundaryCondition.py:126-144 */
int lbm_psi_periodic(const LbmLattice* lat, int32_t axis, void* stream);
/* OpenNeumannPsi / OpenConvective1orderPsi / OpenConvective2orderPsi /
 * OpenExtrapolationPsi .apply — SCBoundaryCondition.py:19-110.  group: psi
 * node coordinates (i, j), halo allowed (-1..NX, -1..NY); the neighbours
 * x - c_direction and x - 2 c_direction must lie on the psi grid, and for the
 * convective kinds x - c_direction inside the lattice (its velocity is
 * averaged over the group). */
enum { LBM_PSI_OPEN_NEUMANN = 0, LBM_PSI_OPEN_CONV1 = 1, LBM_PSI_OPEN_CONV2 = 2, LBM_PSI_OPEN_EXTRAP = 3 };
int lbm_psi_open(const LbmLattice* lat, const int32_t* group, int64_t n, int32_t kind, int32_t direction,
                 void* stream);
/* FixedPsi.apply — SCBoundaryCondition.py:119-123 */
int lbm_psi_fixed(const LbmLattice* lat, const int32_t* group, int64_t n, float value, void* stream);

/* <BoundaryCondition>.apply for every kind in LBM_BC_* —
 * taichi_lbm/BoundaryCondition.py:85-449 (see the enum for each kind's lines) */
int lbm_boundary_apply(const LbmLattice* lat, const LbmBoundary* bc, const int32_t* group,
                       int64_t n, void* stream);

/* ----------------------------------------------------------- multi-component
 * LBField with num_components > 1 (taichi_lbm/lbm.py:5-56) and the
 * two-component Shan-Chen model (ExternalForce.py:66-117).  Arrays are
 * component-major: component c's block follows component c-1's.  The
 * mixture fields (total_rho, total_pressure, vel, temperature) are single. */
#define LBM_MC_MAX 4
typedef struct LbmMCLattice {
  int32_t nx, ny, pitch, psi_pitch;
  int32_t nc;             /* components, 1..LBM_MC_MAX                       */
  float* f;               /* [nc][9][ny][pitch] post-stream populations      */
  float* f2;              /* [nc][9][ny][pitch] post-collision populations   */
  float* rho;             /* [nc][ny][pitch]                                 */
  float* total_rho;       /* [ny][pitch]                                     */
  float* pressure;        /* [nc][ny][pitch]                                 */
  float* total_pressure;  /* [ny][pitch]                                     */
  float* temperature;     /* [ny][pitch]                                     */
  float* vel;             /* [2][ny][pitch] mixture velocity                 */
  float* body_force;      /* [nc][2][ny][pitch]                              */
  float* sc_force;        /* [nc][2][ny][pitch]                              */
  float* psi;             /* [nc][ny+2][psi_pitch] one-node halo             */
  float gravity[2];
} LbmMCLattice;
/* ShanChenForceC2's parameters (ExternalForce.py:67-84): cohesion matrix
 * g_coh, adhesion g_adh per component, the two pseudopotentials (psi_list),
 * and fluid_strategy evaluated on the psi grid: fluid[(j+1)*psi_pitch + i+1]
 * = 1 where fluid_strategy(i, j) holds, for i in -1..NX, j in -1..NY.       */
typedef struct LbmMCShanChen {
  float g_coh[LBM_MC_MAX][LBM_MC_MAX];
  float g_adh[LBM_MC_MAX];
  LbmEos eos[LBM_MC_MAX];
  const uint8_t* fluid;
} LbmMCShanChen;
/* LBField.init_LBM — lbm.py:119-125, every component */
int lbm_mc_init_feq(const LbmMCLattice* lat, const int32_t* group, int64_t n, void* stream);
/* MacroscopicEngine.density — lbm.py:153-164 */
int lbm_mc_density(const LbmMCLattice* lat, const int32_t* group, int64_t n, void* stream);
/* MacroscopicEngine.pressure2 — lbm.py:185-202 */
int lbm_mc_pressure2(const LbmMCLattice* lat, const LbmMCShanChen* sc, const int32_t* group, int64_t n,
                     void* stream);
/* ShanChenForceC2.update_psi — ExternalForce.py:86-92 */
int lbm_mc_update_psi(const LbmMCLattice* lat, const LbmMCShanChen* sc, const int32_t* group, int64_t n,
                      void* stream);
/* PeriodicPsi_LR (axis 0) / PeriodicPsi_BT (axis 1), every component —
 * SCBoundaryCondition.py:126-144 */
int lbm_mc_psi_periodic(const LbmMCLattice* lat, int32_t axis, void* stream);
/* ShanChenForceC2.cau_SCforce — ExternalForce.py:96-117 */
int lbm_mc_sc_force(const LbmMCLattice* lat, const LbmMCShanChen* sc, const int32_t* group, int64_t n,
                    void* stream);
/* MacroscopicEngine.force_density — lbm.py:215-220 */
int lbm_mc_force_density(const LbmMCLattice* lat, const int32_t* group, int64_t n, void* stream);
/* MacroscopicEngine.velocity (mixture) — lbm.py:223-237 */
int lbm_mc_velocity(const LbmMCLattice* lat, const int32_t* group, int64_t n, void* stream);
/* BGKCollision.apply, every component — CollisionEngine.py:96-110;
 * tau: [nc][ny][pitch] relaxation times (BGKCollision.tau) */
int lbm_mc_bgk_apply(const LbmMCLattice* lat, const float* tau, const int32_t* group, int64_t n,
                     void* stream);
/* PeriodicAllBoundary.apply, every component — BoundaryCondition.py:419-432 */
int lbm_mc_stream_periodic(const LbmMCLattice* lat, const int32_t* group, int64_t n, void* stream);

/* ----------------------------------------------------------- fused plan
 * The whole step composed the way the reference's example drivers compose it
 * (cases/Circular cylinder.py:182-193; cases/Power Law Fluid.py:160-173):
 * density -> pressure -> force_density -> velocity -> [shear_rate ->
 * relaxation_time] -> collision.apply -> boundary conditions in insertion
 * order, as ONE pull-scheme kernel per time step.  The fused state is the
 * post-collision population set (f2); launch n streams and applies the
 * boundary conditions of step n-1, then computes the moments and collides
 * step n.  The first collision and the last stream/boundary pass are done by
 * the per-stage kernels above (the host wrapper sequences them).           */

#define LBM_MAX_BC 16
#define LBM_MAX_PROG 64
#define LBM_PROG_LEN 4

/* Per-node code (uint16) of the fused path:
 *  bits 0-7  : link k = bit+1 bounces back (source is the node itself, opposite
 *              population) instead of streaming from (i - cx_k, j - cy_k)
 *  bit 8     : node collides (member of the collision group)
 *  bit 9     : node's moments are saved for next step's boundary conditions
 *  bits 10-15: boundary program id (0 = none), an index into LbmPlanDesc.prog */
#define LBM_CODE_ACTIVE 0x100u
#define LBM_CODE_SAVE 0x200u
#define LBM_CODE_PROG_SHIFT 10

typedef struct LbmPlanDesc {
  int32_t nx, ny, pitch;
  int32_t model;        /* LBM_BGK / LBM_TRT / LBM_MRT                      */
  int32_t fluid_model;  /* LBM_NEWTONIAN / LBM_POWERLAW                     */
  int32_t storage;      /* LBM_STORE_*                                      */
  int32_t nodes_per_thread; /* 1, 2 or 4 (x-consecutive nodes per thread) */
  float tau;            /* Newtonian: uniform tau (BGK) or tau_sym (TRT)    */
  float tau_antisym;    /* Newtonian TRT                                    */
  float magic;          /* TRT magic (power law)                            */
  float tau_min, tau_max, pl_m, pl_n;
  float mrt_s[9];       /* MRT diag (uniform over the collision group)      */
  float gravity[2];     /* body force per node: rho/total_rho * gravity     */
  int32_t nbc;
  LbmBoundary bc[LBM_MAX_BC];      /* rewrite boundaries, velocity_per_node
                                      ignored here (see LbmPlanBuffers)     */
  int32_t nprog;
  int8_t prog[LBM_MAX_PROG][LBM_PROG_LEN]; /* bc indices, -1 terminated     */
  int32_t pipeline;     /* LBM_PIPE_DIRECT: one warp per row segment, vector
                           loads into registers;
                           LBM_PIPE_ASYNC: persistent warps staging source
                           rows through shared memory with cp.async.bulk
                           (needs nodes_per_thread == 4 and a status word);
                           LBM_PIPE_PREFETCH: persistent warps loading the
                           next segment into registers while colliding the
                           current one (nodes_per_thread == 4)             */
  int32_t tune;         /* LBM_PIPE_ASYNC: 0..LBM_ASYNC_TUNINGS-1 selects
                           (warps per block, stages per warp) =
                           (8,2) (6,3) (4,4) (16,2);
                           LBM_PIPE_PREFETCH with a plain list:
                           0..LBM_PREFETCH_TUNINGS-1 selects
                           (8,2) (8,3) (4,4) (16,2) for the plain segments'
                           shared-memory ring                               */
  /* Single-component Shan-Chen (ExternalForce.py:27-63) on a fully periodic
   * lattice: each step computes psi(rho, T) from the post-stream populations,
   * F = -g_coh psi(x) sum_k w_k c_k psi(x + c_k) + gravity, then collides.
   * Needs the direct pipeline, nodes_per_thread 4, no
   * rewrite boundaries and a uniform temperature.                          */
  int32_t sc;
  float g_coh;
  float sc_T;
  LbmEos eos;
  /* 16-bit storages (LBM_STORE_F16S / BF16S / I16S) hold f_k - w_k * rho_ref so the
   * stored value is the small deviation from rest at density rho_ref; choose
   * the lattice's mean density (0 is read as 1).  Ignored for fp32.        */
  float rho_ref;
  /* LBM_STORE_I16S: the step is 2^-fixed_exp, so stored deviations cover
   * |f_k - w_k rho_ref| < 2^(15 - fixed_exp); 0 selects 19 (range 1/16).
   * LBM_FIXED_EXP_MIN..LBM_FIXED_EXP_MAX.  Ignored by other storages.      */
  int32_t fixed_exp;
  /* LBM_PIPE_ASYNC: clock-cycle budget of each wait on a staged copy
   * (0 selects about 2 s).  A wait that runs out sets LBM_STATUS_TIMEOUT;
   * the copies still in flight are then waited for with the default budget
   * before the kernel returns.                                             */
  int64_t wait_cycles;
  /* 1 = in-place (AA-pattern) step: ONE population buffer (bind fa == fb)
   * instead of the ping-pong pair.  Steps alternate two phases whose nodes
   * each read and write the same nine locations: phase A gathers as the
   * pull step does and writes f*_opp(k)(x) where it read f_k(x); phase B
   * reads f_k(x) from slot opp(k) of x and writes f*_k(x) to slot k of x.
   * A run that ends on phase A swaps the streamed pairs back, so between
   * runs the buffer holds what the ping-pong state would hold, bit for bit
   * (that swap is one more pass over the buffer: run many steps per call).
   * Needs the direct pipeline, no Shan-Chen, the lane-granular lists, every
   * bounce-back link cut on both sides (a colliding node that bounces back
   * the population coming from a colliding neighbour is bounced back by it
   * too), no colliding node streaming from a node outside the collision
   * group, and the boundary read sites (LbmPlanBuffers.aa_sites).          */
  int32_t aa;
} LbmPlanDesc;

#define LBM_FIXED_EXP_DEFAULT 19
#define LBM_FIXED_EXP_MIN 12
#define LBM_FIXED_EXP_MAX 22

enum { LBM_PIPE_DIRECT = 0, LBM_PIPE_ASYNC = 1, LBM_PIPE_PREFETCH = 2 };
#define LBM_ASYNC_TUNINGS 4
#define LBM_PREFETCH_TUNINGS 4
/* *status (LbmPlanBuffers.status) is a sticky set of bits that steps OR in
 * and the caller clears:
 *  LBM_STATUS_TIMEOUT    a wait on a staged copy (LBM_PIPE_ASYNC) exceeded
 *                        its budget; the step's output is invalid
 *  LBM_STATUS_SATURATED  LBM_STORE_I16S: a colliding node's post-collision
 *                        value fell outside the fixed-point range (or was
 *                        not finite) and was clamped
 *  LBM_STATUS_NONFINITE  a colliding node's post-collision value was NaN or
 *                        infinite (any storage), or a drag/lift monitor
 *                        summed to a non-finite force
 * Only nodes inside the lattice whose code has LBM_CODE_ACTIVE are checked. */
#define LBM_STATUS_TIMEOUT 1
#define LBM_STATUS_SATURATED 2
#define LBM_STATUS_NONFINITE 4

typedef struct LbmPlanBuffers {
  void* fa;             /* [9][ny][pitch] populations, element type per storage */
  void* fb;
  float* mom_a;         /* [3][ny][pitch] saved (rho, ux, uy)                */
  float* mom_b;
  const uint16_t* code; /* [ny][pitch] node codes                            */
  const uint8_t* seg_flags; /* [ny][nseg] 0 = every node of the segment plain;
                               nseg = ceil(nx / (32 * nodes_per_thread))     */
  const float* bc_vel;  /* [2][ny][pitch] per-node boundary velocity or NULL */
  float* tau;           /* [ny][pitch] power-law state (BGK tau, TRT tau_sym,
                           MRT diag[7]) or NULL                              */
  int32_t* status;      /* one device int32 of LBM_STATUS_* bits; required
                           by LBM_PIPE_ASYNC, optional (NULL) otherwise     */
  /* LBM_PIPE_DIRECT or LBM_PIPE_PREFETCH, optional: the indices (y * nseg + seg, ascending)
   * of every segment whose seg_flags entry is nonzero.  With it a step is two
   * launches, a lean kernel over the plain segments and a general one over
   * the listed segments; NULL keeps one general launch per step.          */
  const int32_t* special;
  int32_t nspecial;
  /* with a special list: 1 = run the listed segments on a plan-owned
   * high-priority stream, forked from the caller's stream by an event before
   * the plain segments are launched and joined back after them, so the two
   * kernels overlap; 0 = both on the caller's stream, one after the other */
  int32_t special_stream;
  /* LBM_PIPE_PREFETCH with a special list: the indices of every segment whose
   * seg_flags entry is zero (ascending).  The plain segments then run on a
   * persistent kernel whose warps load their next segment while colliding
   * the current one.                                                       */
  const int32_t* plain;
  int32_t nplain;
  /* LBM_PIPE_DIRECT with a special list, optional: lane-granular special
   * work.  lane_mask[y * nseg + seg] has bit l set when one of lane l's
   * nodes_per_thread nodes is not plain (bounce-back link, boundary program,
   * saved moments or outside the collision group); lanes lists those lanes
   * as (y * nseg + seg) * 32 + l, ascending.  A step then runs the plain-path
   * kernel on every segment, storing only unmarked lanes, and one thread per
   * listed lane for the rest.                                              */
  const uint32_t* lane_mask;
  const int32_t* lanes;
  int32_t nlanes;
  /* In-place step (LbmPlanDesc.aa): the plane offsets y * pitch + x of every
   * node whose post-stream populations a boundary program reads (the
   * neighbours x - c_dir of VelocityNEEM, PressureNEEM, OpenNeumann and
   * OpenConvective1order nodes, and x - c_dir, x - 2 c_dir of
   * OpenExtrapolation nodes), ascending and distinct, and aa_vals, device
   * scratch of 9 * aa_nsites floats.  Each step gathers those populations
   * into aa_vals before it overwrites them.  Required when a program reads
   * neighbours; ignored by the ping-pong step.                             */
  const int32_t* aa_sites;
  int32_t aa_nsites;
  float* aa_vals;
} LbmPlanBuffers;

typedef struct LbmPlan LbmPlan;

int lbm_plan_create(const LbmPlanDesc* desc, LbmPlan** out);
int lbm_plan_bind(LbmPlan* plan, const LbmPlanBuffers* bufs);
/* Launch nsteps fused steps, alternating fa/fb and mom_a/mom_b (in place:
 * phases A and B on fa, then the swap back after an odd count). */
int lbm_plan_run(LbmPlan* plan, int32_t nsteps, void* stream);
/* Which buffer holds the current post-collision state: 0 = fa/mom_a, 1 = fb/mom_b. */
int lbm_plan_get_parity(const LbmPlan* plan, int32_t* parity);
int lbm_plan_set_parity(LbmPlan* plan, int32_t parity);
/* Stream + boundary conditions of the last step only: writes the post-stream
 * populations (fp32, [9][ny][pitch]) into f_out; moments are not computed.  */
int lbm_plan_stream(LbmPlan* plan, float* f_out, void* stream);
/* Convert fp32 populations into / out of the plan's current state buffer
 * (identity copies for fp32 storage, shifted 16-bit for F16S/BF16S/I16S).
 * Import writes both buffers: a step never writes a node outside the
 * collision group, so fa and fb must hold the same populations there (a
 * caller that fills the buffers itself keeps them equal at those nodes).    */
int lbm_plan_import(LbmPlan* plan, const float* f_post, void* stream);
int lbm_plan_export(LbmPlan* plan, float* f_post, void* stream);
int lbm_plan_destroy(LbmPlan* plan);

/* ----------------------------------------------------------- drag / lift
 * Not in the reference (it has no force evaluation): momentum exchange on
 * half-way bounce-back links into solid nodes.  links holds n pairs
 * (q, k): q = j*pitch + i of a colliding node whose link k points into a
 * solid neighbour (i + cx_k, j + cy_k); the force on the body from the
 * current post-collision state is sum 2 c_k f_k(q), accumulated in FP64 and
 * written to out[0..1] (Fx, Fy). */
int lbm_plan_momentum_exchange(LbmPlan* plan, const int32_t* links, int64_t n, double* out,
                               void* stream);
/* lbm_plan_run followed, after every launch, by the momentum exchange into
 * series[2*s .. 2*s+1] for step s (series holds nsteps x 2 doubles). */
int lbm_plan_run_monitored(LbmPlan* plan, int32_t nsteps, const int32_t* links, int64_t n,
                           double* series, void* stream);

/* ----------------------------------------------------------- reductions
 * FP64 sums over the nodes whose code has LBM_CODE_ACTIVE, of the current
 * population state: out[0] = sum f, out[1] = sum f c_x, out[2] = sum f c_y.
 * partials: caller scratch of at least lbm_reduce_scratch_doubles() doubles. */
int64_t lbm_reduce_scratch_doubles(void);
int lbm_plan_reduce_moments(LbmPlan* plan, double* partials, double* out, void* stream);

/* Allocation-free lbm_plan_reduce_moments (no counterpart in taichi-lbm,
 * which has no reductions at all).  For callers that cannot allocate device
 * memory themselves: a host whose device memory is all handed out by its own
 * pool or budget (a serving loop admitting lattices against an HBM budget
 * has no spare buffer to lend), or a monitor hook between steps that must
 * not trigger cudaMalloc and the device synchronisation it implies.
 * The caller passes only the plan (its bound state is the input) and out.
 * Scratch is a 48 KiB file-scope __device__ array that every GPU which loads
 * the library holds until process exit.  The first call on each device looks
 * its device address up (cudaGetSymbolAddress) with that device current, so
 * make that first call before any stream capture.  The address is kept for
 * the process's life and belongs to the device's primary context (the one
 * the CUDA runtime and PyTorch use): calls from another driver context, or
 * after cudaDeviceReset, are not supported.  Lattices with more than
 * LBM_NOALLOC_MAX_NODES sites (ny * pitch) are rejected with LBM_ERR_ARG
 * before the plan's buffers are looked at, so an unbound plan is rejected
 * the same way.  Every call shares the array: calls that overlap on the GPU
 * race.  No cudaMalloc, cudaFree or allocating library routine is called. */
#define LBM_NOALLOC_CHUNK 16384LL
#define LBM_NOALLOC_MAX_NODES (2048LL * LBM_NOALLOC_CHUNK)
int lbm_plan_reduce_moments_noalloc(LbmPlan* plan, double* out, void* stream);

/* ---------------------------------------------------------------------------
 * Batches: many independent lattices advanced together.  No counterpart in
 * the reference (taichi-lbm steps one LBField per Python loop); the serving
 * and batching layers of this library are built on it.
 *
 * A batch holds bound plans.  lbm_batch_run advances every member nsteps
 * steps: per step, one persistent launch per group of members that share a
 * kernel (plain segments, flagged segments or Shan-Chen tiles x collision
 * model x power law x storage x nodes per thread x body force), walking a
 * packed table of (member, tile) entries, then the members' drag/lift
 * monitors.  Results equal lbm_plan_run on each member alone.  Member plans'
 * parities advance with the batch; a plan must not be run on its own while
 * it is a member.  The batch runs on its own stream, ordered after the
 * caller's stream by an event and joined back to it the same way.  With
 * graphs on, two steps are captured once per membership and replayed.
 * Adding, removing or re-monitoring a member rebuilds the tables at the next
 * run, in stream order (double-buffered tables), without waiting.  The
 * groups of a step run concurrently on the batch's worker streams.         */
typedef struct LbmBatch LbmBatch;
int lbm_batch_create(LbmBatch** out);
/* host_lane_mask: a host copy of the plan's lane_mask ([ny][nseg]), or NULL
 * to read it from the device (a synchronous copy).  Plans other than
 * Shan-Chen ones must be bound with lane masks. */
int lbm_batch_add(LbmBatch* batch, LbmPlan* plan, const uint32_t* host_lane_mask, int32_t* slot);
/* Never waits for the GPU: steps already queued keep reading the member
 * through the previous tables, so its buffers must outlive them (wait for
 * the caller's stream before freeing them). */
int lbm_batch_remove(LbmBatch* batch, int32_t slot);
/* After every step, append the member's momentum-exchange force (Fx, Fy) on
 * its solid links (site, k pairs, as lbm_plan_momentum_exchange) to
 * series[2 * (*count)] while *count < capacity, and increment *count
 * (device int32, set by the caller). */
int lbm_batch_monitor(LbmBatch* batch, int32_t slot, const int32_t* links, int64_t nlinks, double* series,
                      int32_t* count, int32_t capacity);
int lbm_batch_set_graph(LbmBatch* batch, int32_t enable);
/* Members (other than Shan-Chen ones) of at least min_nodes lattice nodes
 * run their own single-lattice step inside each batched step (the plan's
 * lane-granular two-pass launch, parameters by value) instead of the packed
 * tile table; 0 puts every member in the tables.  Default 2^19. */
int lbm_batch_set_solo(LbmBatch* batch, int64_t min_nodes);
/* Rows per Shan-Chen strip (the strip tile is 32 x nodes-per-thread columns
 * by rows): 8, 16 or 32, or 0 for the default (the longest strips that
 * still give every SM several). */
int lbm_batch_set_sc_rows(LbmBatch* batch, int32_t rows);
/* Kernel form of the plain-segment (lean) groups: 0 = one pass per tile, 16
 * tiles per block; 1 = a two-stage cp.async ring per warp, 32 tiles per
 * block; 2 = a three-stage ring, 64 tiles per block.  The pipelined forms
 * keep the next tiles' rows in flight while a warp collides the current one;
 * every form gives the same results to the bit.  Takes effect at the next
 * run (the tables are rebuilt). */
int lbm_batch_set_lean_form(LbmBatch* batch, int32_t form);
int lbm_batch_run(LbmBatch* batch, int32_t nsteps, void* stream);
/* members; tiles and launch units (tile groups and solo members) of the
 * current tables (-1 before the first run after a change) */
int lbm_batch_info(const LbmBatch* batch, int32_t* members, int64_t* tiles, int32_t* groups);
int lbm_batch_destroy(LbmBatch* batch);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
