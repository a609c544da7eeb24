/*
 * pocketwind.h -- C ABI of libpocketwind_gb300, the GB300 (sm_103a) solver hot
 * path of pocketwind: D3Q19 stream-collide with fused momentum-exchange drag,
 * the parity-ray voxelizer, and tracer advection.
 *
 * Every entry point replaces one call of the reference's TypeScript solver
 * interface (intesarjawad/pocketwind); the citation above each declaration
 * names the function it stands in for.  Conventions:
 *   - plain pointers and sizes; caller-owned host output buffers;
 *   - int status returns (PW_OK or a PW_ERR_* code); pw_last_error() holds the
 *     message of the last failure on the calling thread;
 *   - one CUDA stream per domain; a handle is not safe for concurrent use;
 *   - every destroy accepts NULL.
 * Cell n = x + nx*(y + ny*z); populations are reported direction-major,
 * g[i*cells + n], as shifted deviations g = f - w (src/lbm/layout.ts,
 * docs/numerics.md:118-129).
 */
#ifndef POCKETWIND_H
#define POCKETWIND_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PW_API __attribute__((visibility("default")))
#else
#define PW_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  PW_ERR_INVALID stands for the reference's RangeError,
 * PW_ERR_OOM for its AllocationFailure (src/lbm/gpu-resources.ts:3-5),
 * PW_ERR_BUSY for readForce()'s 'busy' (src/lbm/gpu-force.ts:192-194). */
enum {
  PW_OK = 0,
  PW_ERR_INVALID = 1,
  PW_ERR_OOM = 2,
  PW_ERR_UNSTABLE = 3,
  PW_ERR_BUSY = 4,
  PW_ERR_TIMEOUT = 5,
  PW_ERR_CUDA = 6,
  PW_ERR_DESTROYED = 7
};

/* Cell kinds and masks of the packed geometry (src/geometry/voxel-grid.ts:3-5). */
enum { PW_FLUID = 0, PW_SOLID = 1, PW_SUPPORT = 2, PW_FLOOR = 3, PW_EQ = 4 };
#define PW_CELL_TYPE_MASK 7u
#define PW_NO_Q 0xffffffffu

/* Collision operators (src/lbm/params.ts:7) and population storage
 * (src/lbm/layout.ts:5; bf16 is this library's addition). */
enum { PW_OP_TRT = 0, PW_OP_REG = 1 };
enum { PW_WALLS_BB = 0, PW_WALLS_BOUZIDI = 1 };
enum { PW_STORE_F32 = 0, PW_STORE_F16 = 1, PW_STORE_BF16 = 2 };

/* SolverParams (src/lbm/gpu-solver.ts:19-30) plus the layout.  A domain holds
 * up to 2^32 - 64 cells (the reference's shaders stop at 19 x cells < 2^32,
 * 226 M cells; here element indices are 64-bit), PW_KERNEL_TILE up to the
 * reference's limit. */
typedef struct {
  uint32_t nx, ny, nz;
  double tau0;          /* relaxation time; rounded to binary32 like packSolverParams */
  double u_in;          /* inlet speed in lattice units */
  int les;              /* Smagorinsky C_s = 0.1 plus the Werner-Wengle wall cell */
  int op;               /* PW_OP_TRT (Lambda = 3/16) or PW_OP_REG */
  int walls;            /* PW_WALLS_BB (halfway bounce-back) */
  int storage;          /* PW_STORE_F32, PW_STORE_F16 (x2^15, hash-dithered), PW_STORE_BF16 */
  uint32_t ramp_steps;  /* inlet ramp length; 0 starts at full speed (rampFactor, :119-123) */
  int strict;           /* 1: binary32 evaluated in the reference's order without fused
                           multiply-add, so results match a binary32 restatement bit for bit */
  int kernel;           /* PW_KERNEL_AUTO and PW_KERNEL_CELL: one cell per thread (the faster
                           kernel on GB300); PW_KERNEL_TILE: whole x-rows staged through
                           shared memory by bulk copies, which needs nx * element bytes to
                           be a multiple of 16 (PW_ERR_INVALID otherwise) */
  int lateral;          /* PW_LATERAL_PERIODIC (the reference: y and z wrap) or
                           PW_LATERAL_FREE_SLIP (the y and z faces reflect specularly at
                           the halfway plane; no counterpart in the reference) */
} pw_domain_desc;

enum { PW_KERNEL_AUTO = 0, PW_KERNEL_CELL = 1, PW_KERNEL_TILE = 2 };
enum { PW_LATERAL_PERIODIC = 0, PW_LATERAL_FREE_SLIP = 1 };

/* VoxelGrid statistics (src/geometry/voxel-grid.ts:7-15). */
typedef struct {
  uint32_t nx, ny, nz;
  uint32_t solid_cells;
  uint32_t frontal_cells;
  uint32_t watertight;
  uint32_t missed_links;
  uint32_t reserved;
  double blockage;
  uint64_t geometry_len;   /* 2*cells + packed link fractions */
  uint64_t boundary_cells; /* body-adjacent fluid cells */
} pw_grid_stats;

/* ForceSample (src/lbm/gpu-force.ts:11), summed in binary64. */
typedef struct {
  uint64_t step;
  double fx, fy, fz;
} pw_force_sample;

typedef struct pw_grid pw_grid;
typedef struct pw_domain pw_domain;
typedef struct pw_particles pw_particles;
typedef struct pw_streaks pw_streaks;
typedef struct pw_plate_smoke pw_plate_smoke;

/* ---------------------------------------------------------------- misc */
PW_API const char *pw_last_error(void);
PW_API const char *pw_version(void);
/* Number of CUDA devices visible; 0 without a GPU.  Never fails. */
PW_API int pw_device_count(void);

/* ---------------------------------------------------------------- geometry */

/* voxelize(body, supports, layout, {floor, linkFractions:false})
 * (src/geometry/voxelize.ts:172-199, wall-links.ts:99-131) on the GPU:
 * three parity projections with binary64 edge functions, majority vote,
 * EQ/FLOOR boundaries, pull-direction wall masks, q offsets with halfway
 * fractions, and the ascending body boundary list.  Meshes are float32
 * triangle soups (9 floats per triangle) in lattice cells; supports may be
 * NULL.  Returns PW_ERR_INVALID for dims below 2 or non-finite coordinates.
 * The call's temporaries come from the device's default stream-ordered memory
 * pool; the first call raises that pool's release threshold to 256 MB for the
 * process, so later calls reuse the mapped memory. */
PW_API int pw_voxelize(const float *body, uint32_t body_triangles, const float *supports,
                uint32_t support_triangles, uint32_t nx, uint32_t ny, uint32_t nz,
                int floor_on, pw_grid **out);
/* voxelize with opts.linkFractions (voxelize.ts:172-199): link_fractions = 1
 * measures every wall link's fraction as the reference's default does
 * (linkFraction, wall-links.ts:53-80; binTriangles / nearestLinkHit /
 * intersection, triangle-bins.ts:1-162): four-cell triangle bins and one
 * binary64 Moller-Trumbore segment cast per link from the fluid cell toward
 * its wall, nearest hit clamped to [1e-3, 1]; FLOOR links and misses keep 1/2
 * and misses count in pw_grid_stats.missed_links.  link_fractions = 0 is
 * pw_voxelize. */
PW_API int pw_voxelize_opts(const float *body, uint32_t body_triangles, const float *supports,
                            uint32_t support_triangles, uint32_t nx, uint32_t ny, uint32_t nz,
                            int floor_on, int link_fractions, pw_grid **out);

/* A grid from the reference's packed VoxelGrid arrays (geometry = flags,
 * q offsets, f32 fractions; boundary = boundaryCells), validated like
 * validateGeometry (src/lbm/geometry-contract.ts:39-66) and the boundary
 * check of GpuForce.create (src/lbm/gpu-force.ts:76-81). */
PW_API int pw_grid_from_host(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t *geometry,
                      size_t geometry_len, const uint32_t *boundary, size_t nboundary,
                      pw_grid **out);
PW_API int pw_grid_stats_get(const pw_grid *grid, pw_grid_stats *out);
/* Copy the packed geometry (geometry_len words) / boundary list to the host. */
PW_API int pw_grid_read_geometry(const pw_grid *grid, uint32_t *out, size_t capacity);
PW_API int pw_grid_read_boundary(const pw_grid *grid, uint32_t *out, size_t capacity);
PW_API void pw_grid_destroy(pw_grid *grid);

/* ---------------------------------------------------------------- solver */

/* The checks of GpuSolver.create that need no device: packSolverParams
 * (src/lbm/gpu-solver.ts:80-116) throws RangeError before any device work
 * for a grid dimension below 1, a relaxation time that is not above 1/2 after
 * binary32 rounding (0.5 + 2^-26 is not; 0.5 + 2^-24 is), or an inlet speed
 * that is not finite in binary32 (1e100 overflows).  Here also an unknown
 * enumeration or a grid past 2^32 cells.  PW_OK or PW_ERR_INVALID with the
 * message in pw_last_error(); callable without a GPU. */
PW_API int pw_validate_desc(const pw_domain_desc *desc);
/* GpuSolver.create (src/lbm/gpu-solver.ts:158-335): validates the parameters
 * (tau0 > 1/2 after binary32 rounding, finite inlet speed), allocates every
 * buffer or none (PW_ERR_OOM frees partial allocations) and resets to the
 * equilibrium start (init.wgsl). */
PW_API int pw_domain_create(const pw_domain_desc *desc, const pw_grid *grid, pw_domain **out);
/* GpuSolver.destroy (:459-464). */
PW_API void pw_domain_destroy(pw_domain *dom);
/* GpuSolver.reset (:347-355): equilibrium at the start speed in fluid and EQ
 * cells, rest in walls, macros written; drops an unread force sample. */
PW_API int pw_reset(pw_domain *dom);
/* GpuSolver.step(encoder, count, writeMacroOnLast) (:378-395), including the
 * inlet ramp (:401-430).  Work is queued on the domain's stream. */
PW_API int pw_step(pw_domain *dom, uint64_t count, int write_macro_on_last);
/* GpuSolver.stepCount (:342-344). */
PW_API int pw_step_count(const pw_domain *dom, uint64_t *out);
/* GpuSolver.encodeForce (:448-451 / gpu-force.ts:175-189): queue the mean
 * momentum exchange of the two latest states; a pending unread sample makes
 * this a no-op, as the reference's single staging slot does. */
PW_API int pw_encode_force(pw_domain *dom);
/* GpuSolver.readForce (:454-456 / gpu-force.ts:192-205): PW_ERR_BUSY when no
 * encoded sample is pending; otherwise waits for it and returns it. */
PW_API int pw_read_force(pw_domain *dom, pw_force_sample *out);
/* macroBuffer readback: vec4 (rho, ux, uy, uz) per cell, as last written. */
PW_API int pw_read_macros(pw_domain *dom, float *out);
/* The macros of the box [x0, x0 + wx) x [y0, y0 + wy) x [z0, z0 + wz), x
 * fastest, 4 floats per cell, gathered on the GPU: a region of a domain too
 * large to read whole (no counterpart in the reference). */
PW_API int pw_read_macros_box(pw_domain *dom, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t wx, uint32_t wy,
                              uint32_t wz, float *out);
/* queue.writeBuffer(macroBuffer, ...): replace the macro field (4 floats per
 * cell) that the tracers sample, as the reference's particle test does
 * (tests/browser/particles.spec.ts:54-66). */
PW_API int pw_write_macros(pw_domain *dom, const float *in);
/* populationBuffers readback of the latest state: decoded deviations g
 * (binary32, 19*cells), or the stored codes (binary32 bits, or 16-bit codes
 * of f16 x 2^15 / bf16) in the same direction-major order. */
PW_API int pw_read_populations(pw_domain *dom, float *out);
PW_API int pw_read_populations_raw(pw_domain *dom, void *out);
/* No counterpart in the reference.  The same decoded readout as
 * pw_read_populations, but without allocating device memory: for callers that
 * cannot call cudaMalloc when they read the state back (a GPU whose memory is
 * already taken by its domains, or a host that budgets device memory once up
 * front).  pw_read_populations allocates a 19 x cells x 4-byte buffer on first
 * use; this call converts one direction and a slab of z-planes at a time through
 * a fixed 4 MiB array in the library's device image, so nx * ny must be at most
 * 1,048,576 cells (PW_ERR_INVALID otherwise).  CUDA loads that code and array
 * lazily, and loading takes device memory, so pw_domain_create loads them onto
 * its device and looks up the array's address there: create the domain while
 * memory is still free.  The readout's first call on a device repeats the
 * lookup only if that failed, and should come before any stream capture.  The
 * domain's device must be current (PW_ERR_INVALID otherwise).  All calls share
 * the array, so calls that overlap on the GPU race. */
PW_API int pw_read_populations_noalloc(pw_domain *dom, float *out);
/* Replace the latest state (decoded deviations, encoded with the storage's
 * rounding, or raw codes).  Used for initial fields and checkpoint restore. */
PW_API int pw_write_populations(pw_domain *dom, const float *g);
PW_API int pw_write_populations_raw(pw_domain *dom, const void *raw);
/* FP64 totals of the latest state: mass deviation sum(g) and momentum
 * sum(c g) over every non-wall cell. */
PW_API int pw_read_totals(pw_domain *dom, double out[4]);
/* The density guard (src/lbm/nan-guard.ts:39,151-196, nan_guard.wgsl): the
 * stream-collide pass flags any fluid cell whose density is non-finite or
 * outside [0.5, 1.5] on steps that write macros.  Returns the flag of the
 * latest macro step in *unstable, and PW_ERR_TIMEOUT when a staged-row step
 * (PW_KERNEL_TILE) gave up waiting for its copies since that step. */
PW_API int pw_guard_check(pw_domain *dom, int *unstable);
/* injectNaNForRunner (gpu-solver.ts:358-375): a quiet NaN into the rest
 * population of the first fluid cell, written from the host. */
PW_API int pw_inject_nan(pw_domain *dom);
/* Device buffers for interop (macros: float4 per cell; flags: u32 per cell)
 * and the domain's CUDA stream. */
PW_API int pw_domain_buffers(pw_domain *dom, void **macros, void **flags, void **stream);
/* fieldVtkBytes (src/io/field-export.ts:31-33 over writeVtk, src/io/vtk.ts:27-81)
 * for the macros as last written, formatted on the GPU: the 16 * cells + 25
 * bytes that follow writeVtk's header (rho as big-endian binary32, a newline,
 * "VECTORS velocity float\n", velocity * velocity_scale as big-endian binary32
 * triples, a newline).  velocity_scale is latticeToField's speedMps / U_LU
 * (field-export.ts:22-29), a positive finite number; capacity is the size of
 * the host buffer out. */
PW_API int pw_field_vtk_body(pw_domain *dom, double velocity_scale, void *out, size_t capacity);
/* Solver-state checkpoint (the reference has none; its resume restarts cases,
 * scripts/validate.ts).  pw_checkpoint_size gives the blob's byte count;
 * pw_checkpoint_save writes a header (grid size, storage, operator, parameters,
 * step count, checksum), the populations in the storage's own codes, the macros
 * and the force partials; pw_checkpoint_load puts a domain created with the same
 * description and grid back into that state, so that stepping on from it gives
 * the same bits as the run that saved it.  Mismatched, truncated or corrupted
 * blobs are PW_ERR_INVALID and leave the domain as it was. */
PW_API int pw_checkpoint_size(const pw_domain *dom, size_t *bytes);
PW_API int pw_checkpoint_save(pw_domain *dom, void *out, size_t capacity);
PW_API int pw_checkpoint_load(pw_domain *dom, const void *in, size_t size);
/* Time count steps on the domain's stream with CUDA events; *ms receives the
 * elapsed device time. */
/* ---- batches: many independent domains stepped together (no reference counterpart;
   the reference runs one solver at a time, src/app/solver-slot.ts) ----
   Members are domains of the fast build's one-cell-per-thread path sharing
   storage, operator and LES, with equal step counts and no ramp in progress.
   Each batch step is two persistent launches, one over all members' plain
   cells and one over their seam and edge cells running beside it, replayed
   from captured CUDA graphs; members keep their own force, macro and readout
   calls, which wait for the batch's queued steps.  A member must not be
   stepped on its own while it belongs to a batch. */
typedef struct pw_batch pw_batch;
typedef struct {
  uint32_t blocks;         /* persistent grid chosen */
  uint32_t rows_per_item;  /* plain rows per work item chosen */
  float ms_per_step;       /* its measured time per step */
  uint32_t candidates;     /* launch shapes timed */
} pw_batch_tuning;
PW_API int pw_batch_create(pw_domain *const *members, uint32_t count, pw_batch **out);
PW_API void pw_batch_destroy(pw_batch *batch);
PW_API int pw_batch_step(pw_batch *batch, uint64_t count, int write_macro_on_last);
PW_API int pw_batch_time_steps(pw_batch *batch, uint64_t count, float *ms);
/* Autotuner: times each candidate shape over trial_steps real steps (they
   advance the members) and keeps the fastest. */
PW_API int pw_batch_tune(pw_batch *batch, uint32_t trial_steps, pw_batch_tuning *out);
/* pw_reset of every member; the batch starts again at step 0. */
PW_API int pw_batch_reset(pw_batch *batch);

/* ---- the learned subgrid closure (no counterpart in the reference) ----
   A 9 -> 32 -> 32 -> 1 network scales the Smagorinsky eddy viscosity of plain
   LES cells by max(0, 1 + c); c = 0 (the untrained network) is Smagorinsky.
   Parameters: W1[32][9] b1[32] W2[32][32] b2[32] W3[32] b3 (1409 floats),
   bfloat16 in the forward pass with binary32 accumulation. */
typedef struct pw_closure pw_closure;
#define PW_CLOSURE_PARAMS 1409
#define PW_CLOSURE_INPUTS 9
PW_API int pw_closure_create(uint64_t seed, pw_closure **out);
PW_API void pw_closure_destroy(pw_closure *c);
PW_API int pw_closure_get_params(pw_closure *c, float *out);
PW_API int pw_closure_set_params(pw_closure *c, const float *in);
/* network outputs for count input rows (9 floats each), the fused kernel's path */
PW_API int pw_closure_eval(pw_closure *c, const float *x, uint32_t count, float *out);
/* one forward and backward pass over count samples: parameter gradients of the
   mean squared error, and that error */
PW_API int pw_closure_gradients(pw_closure *c, const float *x, const float *y, uint32_t count, float *grad,
                                float *loss);
/* training data: samples from a fine domain's latest macros, box-filtered 2x
   onto the coarse grid whose molecular viscosity is nu0_coarse */
PW_API int pw_closure_dataset_add(pw_closure *c, pw_domain *fine, double nu0_coarse, uint64_t *added);
PW_API int pw_closure_dataset_clear(pw_closure *c);
PW_API int pw_closure_dataset_reserve(pw_closure *c, uint64_t capacity);
PW_API int pw_closure_dataset_write(pw_closure *c, const float *x, const float *y, uint64_t count);
PW_API int pw_closure_dataset_size(const pw_closure *c, uint64_t *n);
PW_API int pw_closure_dataset_read(pw_closure *c, uint64_t first, uint64_t count, float *x, float *y);
/* Adam (lr, betas 0.9 / 0.999) over `steps` minibatches drawn by a seeded hash */
PW_API int pw_closure_train(pw_closure *c, uint32_t steps, uint32_t batch, float lr, uint64_t seed,
                            float *loss_first, float *loss_last);
/* Attach (c) or detach (NULL) a closure to an LES domain of the fast build; the
   domain restarts from its initial state.  The closure must outlive the attachment.
   The closure acts on the plain fluid cells; the wall-link cells keep plain
   Smagorinsky and the wall model.  A domain with a closure attached cannot join
   a batch (PW_ERR_INVALID). */
PW_API int pw_closure_attach(pw_domain *dom, const pw_closure *c);

PW_API int pw_time_steps(pw_domain *dom, uint64_t count, float *ms);
/* Queue `count` steps (no graphs) with CUDA events around each launch class and
   sum their device times: kernel_ms[0] the plain-cell kernel, [1] its seam-row
   variant (odd steps), [2] the edge-cell kernel.  Outside the fast build's
   one-cell-per-thread path the whole step counts as [0].  No counterpart in the
   reference (a measurement aid). */
PW_API int pw_profile_steps(pw_domain *dom, uint64_t count, float kernel_ms[3]);

/* ---------------------------------------------------------------- tracers */

/* particles_update.wgsl (src/render/particles.ts, particle-layout.ts): 3-D
 * trilinear velocity from the domain's macros, capped Euler step, hash
 * respawn at x = 2.  Records are 8 floats (pos.xyz, age, prev.xyz, generation). */
PW_API int pw_particles_create(pw_domain *dom, const float *records, uint32_t count, uint32_t seed,
                        const float cross_section[4], const float fallback[2],
                        pw_particles **out);
PW_API int pw_particles_update(pw_particles *p, float steps);
PW_API int pw_particles_read(pw_particles *p, float *out);
PW_API int pw_particles_write(pw_particles *p, const float *records);
PW_API void pw_particles_destroy(pw_particles *p);

/* plate_smoke.wgsl (src/render/plate.ts:136-139,218-240,522-548,
 * plate-layout.ts:104-130): rake threads plus dye ports on one y plane, ring of
 * slots per thread, RK2 bilinear advection with slide and settle.  Records are
 * vec4 (x, z, release index, density). */
PW_API int pw_plate_create(pw_domain *dom, uint32_t plane, uint32_t rake_threads, uint32_t slots,
                    const float *ports, uint32_t nports, pw_plate_smoke **out);
PW_API int pw_plate_advance(pw_plate_smoke *s, uint32_t release, int releasing, const float rake[4]);
PW_API int pw_plate_read(pw_plate_smoke *s, float *out);
PW_API void pw_plate_destroy(pw_plate_smoke *s);

/* 3-D streaklines: a ry x rz rake at x = rake[0] spanning y in [rake[1],
 * rake[2]] and z in [rake[3], rake[4]], a ring of `slots` puffs per nozzle,
 * trilinear RK2 with plate_smoke's sub-step, cap, slide and settle rules.
 * Records are vec4 (x, y, z, density) plus a u32 release index per slot. */
PW_API int pw_streaks_create(pw_domain *dom, uint32_t ry, uint32_t rz, uint32_t slots,
                      const float rake[5], pw_streaks **out);
PW_API int pw_streaks_advance(pw_streaks *s, float h_steps, uint32_t release, int releasing);
PW_API int pw_streaks_read(pw_streaks *s, float *puffs, uint32_t *release_of);
PW_API void pw_streaks_destroy(pw_streaks *s);

#ifdef __cplusplus
}
#endif
#endif /* POCKETWIND_H */
