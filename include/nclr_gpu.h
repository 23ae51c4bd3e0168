/*
 * nclr_gpu.h -- C ABI of the GB300 MLS-MPM step (libnclr_gpu.so).
 *
 * The reference exposes its step only as the header-only C++ class template
 * nclr::MPMSimulation<dim> (src/nclr.h:63-384); it has no FFI of its own.  These entry
 * points are what a binding of that class needs, one per member it offers:
 *
 *   nclr_create          MPMSimulation(particles, model, res, dt, E, nu, gravity)
 *                          src/nclr.h:74-78 (and Particle<dim>, src/nclr.h:20-48)
 *   nclr_advance         advance()                    src/nclr.h:80-84
 *   nclr_get_particles   particles()                  src/nclr.h:86
 *   nclr_get_grid        grid()                       src/nclr.h:87
 *   nclr_get_lame        mu_0, lambda_0               src/nclr.h:71-72,77-78
 *   nclr_destroy         ~MPMSimulation()
 *   nclr_last_error      (errors: the reference throws std::out_of_range from vector::at,
 *                          src/nclr.h:163-164,199; here a status code plus a message)
 *
 * plus nclr_set_particles (replace the particle state in place, for embedders that edit
 * particles between steps) and device-pointer variants for callers whose data already
 * lives on the GPU.  include/nclr.h wraps all of this back into the reference's C++ API.
 *
 * Host array layout (particle-major, matrices row-major):
 *   x[p*dim + d], v[p*dim + d], F[(p*dim + r)*dim + c], C likewise, Jp[p], mass[p],
 *   volume[p].  Grid: velocity[node*dim + d], mass[node], node = (i*(res+1) + j)*(res+1) + k
 *   in 3D and i*(res+1) + j in 2D (the reference's index, src/nclr.h:141-142,152).
 *
 * Conventions: every call returns an nclr_status; no exception crosses the ABI.  A handle
 * owns one CUDA stream and its device memory; calls on one handle must not overlap.
 */
#ifndef NCLR_GPU_H
#define NCLR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nclr_status {
  NCLR_OK = 0,
  NCLR_ERR_INVALID = 1,      /* bad argument (null handle, dim not 2/3, res < 1, ...) */
  NCLR_ERR_OUT_OF_RANGE = 2, /* a particle's stencil left the grid: the reference's
                                std::out_of_range (src/nclr.h:163-164,199) */
  NCLR_ERR_CUDA = 3,         /* a CUDA runtime error (message in nclr_last_error) */
  NCLR_ERR_NO_DEVICE = 4     /* no usable CUDA device */
} nclr_status;

/* MaterialModel, src/nclr.h:57-61 */
enum { NCLR_SNOW = 0, NCLR_JELLY = 1, NCLR_LIQUID = 2 };

/* Physics mode.  NCLR_PHYSICS_REFERENCE reproduces the reference bit-for-bit in
 * semantics, including diag<3>(1) == diag(1,1,0) (src/nclr_math.h:13-19) and the 2D SVD
 * sign fix being a no-op (src/nclr_math.h:63-71 write out of bounds in 2D).
 * NCLR_PHYSICS_CORRECTED uses the true identity and applies the 2D sign fix to column 1. */
enum { NCLR_PHYSICS_REFERENCE = 0, NCLR_PHYSICS_CORRECTED = 1 };

/* Stress model.  NCLR_STRESS_COROTATED is the reference's fixed-corotated stress
 * (first_piola_kirchoff_stress, src/nclr.h:313-337): Kirchhoff stress
 * 2 mu (F - R) F^T + constmat(lambda (J - 1) J).  NCLR_STRESS_NEOHOOKEAN is the model the
 * reference lists as a TODO (src/nclr.h:339): mu (F F^T - I) + lambda ln(J) I, with the same
 * hardening of mu and lambda and the same plasticity; it needs det F > 0, so 3D takes it only
 * with NCLR_PHYSICS_CORRECTED (the reference's diag<3>(1) = diag(1,1,0) keeps det F at 0). */
enum { NCLR_STRESS_COROTATED = 0, NCLR_STRESS_NEOHOOKEAN = 1 };

typedef struct nclr_options {
  int physics;             /* NCLR_PHYSICS_* (default REFERENCE) */
  int sort_interval;       /* re-sort particles by grid block every this many steps (0 = only
                              after an upload; default 8) */
  int p2g_particles_per_thread; /* particles per thread of the small-scene kernel (it launches
                              ceil(n / (256 * this)) CTAs; default 1); the tile path steps one
                              particle per thread */
  int device;              /* CUDA device ordinal (default 0) */
  int use_graphs;          /* capture advance() step sequences in CUDA graphs (default 1) */
  int profile;             /* time every kernel phase of advance() with CUDA events on the
                              handle's stream (direct launches, no graphs; default 0) */
  int graph_steps;         /* steps per captured CUDA graph, rounded up to a multiple of
                              sort_interval (0 = one sort interval; default 0) */
  int sparse_block_max;    /* grid blocks holding fewer particles than this (at the last sort)
                              are stepped particle by particle, gathering from and scattering
                              into the grid directly instead of through a shared-memory tile;
                              0 = never, -1 = the default (default -1: 64 in 3D and 32 in 2D
                              for one simulation, 32 for a batch) */
  int small_scene_max;     /* simulations of at most this many particles (per scene) run all
                              the steps of an advance() call in one kernel launch (reference
                              order p2g / grid_op / g2p, grid-wide barriers: one scene that
                              fits a thread-block cluster runs as one and uses its hardware
                              barrier, others a cooperative launch; a batch gives each scene
                              its own group of CTAs) instead of two launches per step;
                              0 = never, -1 = automatic (default -1: one
                              scene of at most 65,536 particles in 2D or 32,768 in 3D whose grid
                              has at most 8 nodes per particle -- that kernel updates every
                              node each step; never a batch, where the tile path is faster) */
  int stress_model;        /* NCLR_STRESS_* (default COROTATED); a batch's scenes share it */
  int batch_item_threads;  /* batches: threads that step one grid block of the fused step
                              together -- 128 (half a CTA, each half with its own tiles; the
                              2D default) or 256 (a whole CTA; the 3D one); 0 = the default.
                              An autotuner knob: the best size depends on the particles per
                              block. */
  int tail_max;            /* one simulation: a grid block of more than 256 particles (at the
                              last sort) steps them in passes of 256 through its tiles; when
                              its last pass would hold fewer than this many, those particles
                              are stepped particle by particle like a thin block's instead, so
                              that no pass runs a few particles while the rest of the CTA
                              waits.  0 = never, -1 = the default (64); batches never */
} nclr_options;

/* Kernel phases reported by nclr_profile_get: the block sort of the particles, the grid
 * update sweep (grid_op + clearing the accumulator), the stand-alone P2G that follows an
 * upload, and the fused G2P + next-step P2G kernel that makes up the rest of a step.  The
 * last three are the reverse kernels of a rollout's backward pass (nclr_rollout_profile_get):
 * the adjoint of G2P, of the grid update, and of P2G.  The last is the FP64 recomputation of
 * the snow clamps that the fused kernel flags as ill-conditioned in FP32. */
enum { NCLR_PHASE_SORT = 0, NCLR_PHASE_GRID = 1, NCLR_PHASE_P2G = 2, NCLR_PHASE_G2P2G = 3,
       NCLR_PHASE_ADJ_G2P = 4, NCLR_PHASE_ADJ_GRID = 5, NCLR_PHASE_ADJ_P2G = 6,
       NCLR_PHASE_SNOW_FIX = 7, NCLR_NUM_PHASES = 8 };

typedef struct nclr_sim nclr_sim;

/* Fills *opt with the defaults. */
void nclr_default_options(nclr_options *opt);

/* One scene of a batch: the arguments of nclr_create for one simulation (same layouts, NULL
 * rules and meaning). */
typedef struct nclr_scene {
  int64_t n;
  const float *x, *v, *F, *C, *Jp, *mass, *volume; /* HOST arrays */
  const uint8_t *material;                         /* NULL = every particle uses `model` */
  int model;
  int res;
  float dt, E, nu, gravity;
} nclr_scene;

/* Creates a simulation of n particles (MPMSimulation ctor, src/nclr.h:74-78).  x, v, F, C,
 * Jp, mass, volume are HOST arrays in the layout above; v, C may be NULL (zero), F NULL
 * (diag<dim>(1) of the chosen physics), Jp/mass/volume NULL (1).  material may be NULL
 * (every particle uses `model`) or hold one NCLR_* value per particle (an extension: the
 * reference has one material per simulation).  opt may be NULL (defaults). */
nclr_status nclr_create(nclr_sim **out, int dim, int64_t n, const float *x, const float *v,
                        const float *F, const float *C, const float *Jp, const float *mass,
                        const float *volume, const uint8_t *material, int model, int res,
                        float dt, float E, float nu, float gravity, const nclr_options *opt);

/* nclr_create with DEVICE arrays (same layouts and NULL rules): scenes built or kept on the
 * GPU are not staged through the host.  An extension. */
nclr_status nclr_create_device(nclr_sim **out, int dim, int64_t n, const float *x, const float *v,
                               const float *F, const float *C, const float *Jp, const float *mass,
                               const float *volume, const uint8_t *material, int model, int res,
                               float dt, float E, float nu, float gravity,
                               const nclr_options *opt);

/* Scene builders on the device.  nclr_cube_device writes cube<dim>(res, lo, hi)
 * (src/nclr_math.h:100-129: res^dim lattice points over [lo, hi]^dim from Eigen's
 * LinSpaced, x outermost) as res^dim rows of dim floats into the DEVICE array x, bit-equal
 * to the host builder.  nclr_cubes_device writes ncubes such lattices one after another,
 * cube c over [lo[c], hi[c]] (HOST arrays) -- the headless solver's generate_cubes
 * (src/solver.cpp:133-149).  Both run on `stream` (a cudaStream_t, NULL = default) and
 * synchronise it. */
nclr_status nclr_cube_device(int dim, int res, float lo, float hi, float *x, void *stream);
nclr_status nclr_cubes_device(int dim, int ncubes, int res, const float *lo, const float *hi,
                              float *x, void *stream);

/* Batched form (no counterpart in the reference, which runs one simulation per object): one
 * handle holding `nscenes` independent simulations of uneven particle counts, grid
 * resolutions, materials and parameters, stepped together -- every kernel of a step covers
 * all scenes in one launch.  nclr_advance steps every scene (each with its own dt); the
 * per-scene functions below read and write one scene; nclr_get_particles / nclr_set_particles
 * address all scenes concatenated in scene order; nclr_get_grid returns scene 0's grid. */
nclr_status nclr_batch_create(nclr_sim **out, int dim, int nscenes, const nclr_scene *scenes,
                              const nclr_options *opt);
int nclr_num_scenes(const nclr_sim *sim);
nclr_status nclr_scene_get_particles(nclr_sim *sim, int scene, float *x, float *v, float *F,
                                     float *C, float *Jp);
nclr_status nclr_scene_set_particles(nclr_sim *sim, int scene, const float *x, const float *v,
                                     const float *F, const float *C, const float *Jp);
nclr_status nclr_scene_get_grid(nclr_sim *sim, int scene, float *velocity, float *mass);
/* NCLR_ERR_OUT_OF_RANGE if a stencil of `scene` left its grid during the last nclr_advance. */
nclr_status nclr_scene_status(const nclr_sim *sim, int scene);

/* advance() repeated nsteps times (src/nclr.h:80-84).  Returns NCLR_ERR_OUT_OF_RANGE if any
 * stencil left the grid during these steps (the state is then unspecified, as the
 * reference's is after its exception).  Synchronises the handle's stream once at the end. */
nclr_status nclr_advance(nclr_sim *sim, int64_t nsteps);

/* particles() (src/nclr.h:86): copies the state, in the caller's original particle order,
 * into HOST arrays (any may be NULL to skip that field). */
nclr_status nclr_get_particles(nclr_sim *sim, float *x, float *v, float *F, float *C, float *Jp);

/* Replaces the particle state (HOST arrays, same layout and NULL rules as nclr_get_particles;
 * a NULL field keeps its current value).  Particle count and order are the caller's. */
nclr_status nclr_set_particles(nclr_sim *sim, const float *x, const float *v, const float *F,
                               const float *C, const float *Jp);

/* Per-particle Young's modulus and Poisson ratio (an extension: the reference has one pair per
 * simulation, src/nclr.h:74-78).  E and nu hold one value per particle in the caller's order
 * (all scenes concatenated for a batch); every particle's mu_0 and lambda_0 then follow from
 * its own pair by the constructor's formula (src/nclr.h:77-78), and the material's hardening
 * scales them as before.  Both NULL returns to the simulation's (each scene's) E and nu.  Takes
 * effect from the next advance(); the values stay with their particles.  nclr_set_moduli takes
 * HOST arrays and synchronises; nclr_set_moduli_device takes DEVICE arrays, ordered on the
 * handle's stream. */
nclr_status nclr_set_moduli(nclr_sim *sim, const float *E, const float *nu);
nclr_status nclr_set_moduli_device(nclr_sim *sim, const float *E, const float *nu);

/* grid() (src/nclr.h:87): the post-update grid of the last step, (res+1)^dim nodes, in the
 * reference's node order.  Before the first advance the reference's grid is empty: returns
 * NCLR_ERR_INVALID then. */
nclr_status nclr_get_grid(nclr_sim *sim, float *velocity, float *mass);

/* Device-pointer variants: same layouts, pointers into device memory of the handle's
 * device.  They are ordered on the handle's stream and return without synchronising. */
nclr_status nclr_get_particles_device(nclr_sim *sim, float *x, float *v, float *F, float *C,
                                      float *Jp);
nclr_status nclr_set_particles_device(nclr_sim *sim, const float *x, const float *v,
                                      const float *F, const float *C, const float *Jp);
/* grid() into device arrays (scene 0), ordered on the handle's stream. */
nclr_status nclr_get_grid_device(nclr_sim *sim, float *velocity, float *mass);

/* Headless renderer (replaces the reference's X11 canvas, src/solver.cpp:184-201): draws
 * n particles (DEVICE rows x of dim floats; 3D is drawn in the x-y plane) as discs of
 * `radius` pixels over the canvas background and boundary box into the DEVICE array rgba
 * (width*height 0xRRGGBB values, row 0 at the top, y up in the scene).  colors (DEVICE, one
 * per particle, the Particle's c) may be NULL: every particle then takes `color`.  Particles
 * are painted in index order.  Ordered on `stream` (a cudaStream_t, NULL = default). */
nclr_status nclr_render_device(const float *x, int64_t n, int dim, const uint32_t *colors,
                               uint32_t color, int width, int height, float radius,
                               uint32_t *rgba, void *stream);

/* Public constants of the simulation (src/nclr.h:66-72). */
nclr_status nclr_get_lame(const nclr_sim *sim, float *mu_0, float *lambda_0);

/* Sizes: particle count, dimension, grid resolution, grid node count. */
int64_t nclr_num_particles(const nclr_sim *sim);
int nclr_dim(const nclr_sim *sim);
int nclr_res(const nclr_sim *sim);
int64_t nclr_num_nodes(const nclr_sim *sim);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their own work on it. */
void *nclr_stream(nclr_sim *sim);

/* Counters of the last nclr_advance call: number of kernel launches it enqueued, and the
 * number of grid nodes that received mass in its last step (0 if not tracked). */
nclr_status nclr_stats(const nclr_sim *sim, int64_t *kernel_launches, int64_t *active_nodes);

/* Number of grid nodes holding mass after the last step's P2G (a reduction over the grid). */
nclr_status nclr_count_active_nodes(nclr_sim *sim, int64_t *active_nodes);

/* With opt.profile set: accumulated device time (ms, CUDA events on the handle's stream) and
 * launch count of one kernel phase over all advance() calls since the last reset. */
nclr_status nclr_profile_get(const nclr_sim *sim, int phase, double *total_ms, int64_t *launches);
nclr_status nclr_profile_reset(nclr_sim *sim);

/* Test hook for the small-scene kernels' grid barrier (the one-launch-per-call path, single
 * scenes and batches), which gives up a wait after a bounded number of polls (about a second)
 * and reports it.  With extra_arrivals > 0 every barrier waits for that many CTAs beyond the
 * launch's, which never come, so each wait runs out after spin_limit polls (~64 ns each;
 * 0 = the default limit): the call returns NCLR_ERR_CUDA ("grid barrier ran out of time"),
 * leaves the particle state half stepped and the handle usable.  (0, 0) restores the normal
 * barrier.  No counterpart in the reference. */
nclr_status nclr_debug_set_barrier(nclr_sim *sim, unsigned extra_arrivals, unsigned spin_limit);

/* Message of the last failed call on this handle ("" if none); valid until the next call.
 * With sim == NULL: the last failure of nclr_create on this thread. */
const char *nclr_last_error(const nclr_sim *sim);

void nclr_destroy(nclr_sim *sim);

/* ---------------------------------------------------------------------------------------
 * Differentiable rollouts (no counterpart in the reference).  A rollout is `nsteps` steps
 * (src/nclr.h:80-372) of one material from a given state; the reverse pass is a hand-written
 * adjoint of the whole step (G2P with the material's plasticity -- the snow clamp through the
 * derivative of its singular values and the Jp update, the liquid reset through det F --, grid
 * update with its clamp and boundary masks, P2G, the hardening, the stress of
 * opt->stress_model -- fixed corotated with its polar rotation, or neo-Hookean) run backwards
 * through the rollout, recomputing each segment of `checkpoint_every` steps from a checkpoint.
 * Jp is part of the state (1 at the start, as Particle<dim> sets it); nothing is read of the
 * final Jp, so its adjoint starts at zero.
 *
 * All state arrays are DEVICE pointers in the host layout above (caller order, rows).
 * nclr_rollout_create takes the particle count, initial positions (HOST, used only to size and
 * place the simulation), mass and volume (HOST, NULL = 1) and the step constants;
 * nclr_rollout_forward runs from (x0, v0, F0, C0) with the given E and nu (Jp = 1) and writes
 * the final state (any output may be NULL); nclr_rollout_backward takes the adjoint of the
 * final state (NULL = 0) and writes the adjoint of the initial state (outputs may be NULL) and
 * of E and nu.  Calls are ordered on the rollout's stream and synchronise it before
 * returning. */
typedef struct nclr_rollout nclr_rollout;
nclr_status nclr_rollout_create(nclr_rollout **out, int dim, int64_t n, const float *x0,
                                const float *mass, const float *volume, int res, float dt,
                                float gravity, int64_t nsteps, int checkpoint_every,
                                const nclr_options *opt);
/* The same for any material model (NCLR_SNOW, NCLR_JELLY, NCLR_LIQUID); nclr_rollout_create is
 * this with NCLR_JELLY. */
nclr_status nclr_rollout_create_model(nclr_rollout **out, int dim, int64_t n, const float *x0,
                                      const float *mass, const float *volume, int model, int res,
                                      float dt, float gravity, int64_t nsteps,
                                      int checkpoint_every, const nclr_options *opt);
nclr_status nclr_rollout_forward(nclr_rollout *r, const float *x0, const float *v0, const float *F0,
                                 const float *C0, float E, float nu, float *xT, float *vT,
                                 float *FT, float *CT);
nclr_status nclr_rollout_backward(nclr_rollout *r, const float *gxT, const float *gvT,
                                  const float *gFT, const float *gCT, float *gx0, float *gv0,
                                  float *gF0, float *gC0, double *gE, double *gnu);
/* The same with one Young's modulus and Poisson ratio per particle (the extension of
 * nclr_set_moduli): E and nu are DEVICE arrays of n values in row order.  The matching
 * backward writes the adjoint of every particle's E and nu into the DEVICE arrays gE, gnu
 * (n values each, may be NULL).  A backward must match its forward: after
 * nclr_rollout_forward_moduli only nclr_rollout_backward_moduli, after nclr_rollout_forward
 * only nclr_rollout_backward (NCLR_ERR_INVALID otherwise). */
nclr_status nclr_rollout_forward_moduli(nclr_rollout *r, const float *x0, const float *v0,
                                        const float *F0, const float *C0, const float *E,
                                        const float *nu, float *xT, float *vT, float *FT,
                                        float *CT);
nclr_status nclr_rollout_backward_moduli(nclr_rollout *r, const float *gxT, const float *gvT,
                                         const float *gFT, const float *gCT, float *gx0,
                                         float *gv0, float *gF0, float *gC0, float *gE,
                                         float *gnu);
/* Device time (ms, CUDA events on the rollout's stream) of the last forward and backward. */
nclr_status nclr_rollout_timing(const nclr_rollout *r, double *forward_ms, double *backward_ms);
/* With nclr_options.profile set at creation: per kernel phase (NCLR_PHASE_*), the device time
 * and launch count since the last reset -- the forward kernels of the forward pass and of the
 * backward's recomputation, and the three reverse kernels of every backward step, each timed
 * with CUDA events on the stream it runs on.  Profiling launches the forward without graphs. */
nclr_status nclr_rollout_profile_get(const nclr_rollout *r, int phase, double *total_ms,
                                     int64_t *launches);
nclr_status nclr_rollout_profile_reset(nclr_rollout *r);
void *nclr_rollout_stream(nclr_rollout *r);
/* Message of the rollout's last failed call; with r == NULL the last nclr_rollout_create
 * failure of this thread. */
const char *nclr_rollout_error(const nclr_rollout *r);
void nclr_rollout_destroy(nclr_rollout *r);

/* ---------------------------------------------------------------------------------------
 * Particle-to-grid transfer without any allocation.  No counterpart in the reference: it is
 * an addition for callers that cannot call cudaMalloc while they run -- applications whose
 * own allocator already holds the device's memory, real-time loops where allocating (and the
 * synchronisation it can imply) is not allowed, plugins inside a runtime that owns every
 * allocation.  Everything else in this header allocates in nclr_create.
 *
 * Computes the reference's p2g() + grid_op() (src/nclr.h:104-165, 263-310) -- the grid that
 * grid() returns after one advance() from this state -- for n particles in the caller's
 * DEVICE memory (the host layout above: x[p*dim+d], F[(p*dim+r)*dim+c], ...; all seven
 * arrays required) into the caller's DEVICE arrays grid_velocity[(res+1)^dim * dim] and
 * grid_mass[(res+1)^dim], in the reference's node order.  Runs on `stream` (a cudaStream_t,
 * NULL = legacy default stream) of the calling thread's current device; every call copies its
 * error flag back and synchronises that stream before returning.
 *
 * What it computes: the fixed-corotated stress of src/nclr.h:313-337 with one material
 * (`model`), one E and one nu for every particle -- no per-particle materials or moduli and no
 * neo-Hookean option.  The physics mode of nclr_options does not change this transfer (the
 * diag(1,1,0) identity and the 2D SVD sign fix enter only G2P), so the grid equals grid()
 * after one nclr_advance under either mode.
 *
 * The only memory it uses beyond the caller's arrays is a static device array of
 * NCLR_NOALLOC_MAX_NODES float4 nodes (16 MiB) in the library, held by every GPU that loads
 * the library until the process exits.  So (res+1)^dim must not exceed
 * NCLR_NOALLOC_MAX_NODES (3D: res <= 100; 2D: res <= 1023): larger grids return
 * NCLR_ERR_INVALID.  The array is shared by all calls and keeps the last call's contents;
 * each call clears it before use.  Calls whose GPU work overlaps (other threads or streams at
 * the same time) race on it: serialise them (the library does not).  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and keeps it for the
 * context it was made in; a call in another context of the device (after cudaDeviceReset, or
 * in a caller's own context) looks the address up again.  No call can run inside a stream
 * capture: each one reads its status back and synchronises its stream.  Errors:
 * NCLR_ERR_INVALID (bad argument, grid too large), NCLR_ERR_OUT_OF_RANGE (a
 * stencil left the grid, the reference's std::out_of_range), NCLR_ERR_CUDA; when `message`
 * is non-NULL, up to message_len - 1 bytes of explanation are written there.
 * --------------------------------------------------------------------------------------- */
#define NCLR_NOALLOC_MAX_NODES (1 << 20)
nclr_status nclr_grid_transfer_noalloc(int dim, int64_t n, const float *x, const float *v,
                                       const float *F, const float *C, const float *Jp,
                                       const float *mass, const float *volume, int model,
                                       int res, float dt, float E, float nu, float gravity,
                                       float *grid_velocity, float *grid_mass, void *stream,
                                       char *message, size_t message_len);

#ifdef __cplusplus
}
#endif

#endif /* NCLR_GPU_H */
