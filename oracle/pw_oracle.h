/*
 * pw_oracle.h -- CPU oracle for the pocketwind solver hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, and only as the checker.
 *
 * Four independent restatements of the reference (intesarjawad/pocketwind),
 * each pinned by the reference's own unit-test golden values (tests/):
 *   ow_*  FP32 restatement of the WGSL stream-collide, init and force kernels
 *         (the .wgsl files in src/lbm/shaders) with the reference's A/B ping-pong pull
 *         scheme, evaluated statement for statement in IEEE binary32
 *         (compiled with -ffp-contract=off so no multiply-add is fused).
 *   oc_*  FP64 restatement of the TypeScript CpuSolver
 *         (src/lbm/reference/cpu-solver.ts, collision.ts).
 *   ov_*  FP64 restatement of the voxelizer and wall-link packer
 *         (src/geometry/voxelize.ts, wall-links.ts, triangle-bins.ts).
 *   ot_*  FP32 restatement of the tracer kernels
 *         (src/render/shaders/particles_update.wgsl, plate_smoke.wgsl) and of
 *         this project's 3-D streakline rule built from them.
 */
#ifndef PW_ORACLE_H
#define PW_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- storage codecs (src/lbm/shaders/prelude-f16.wgsl:7-22) ---- */
uint16_t ow_f32_to_f16_rne(float f);
float ow_f16_to_f32(uint16_t h);
uint16_t ow_f32_to_bf16_rne(float f);
float ow_bf16_to_f32(uint16_t h);
uint16_t ow_encode_f16(float scaled, uint32_t i, uint32_t n);
uint16_t ow_encode_bf16(float value, uint32_t i, uint32_t n);

/* ---- FP32 WGSL restatement ---- */
typedef struct ow_solver ow_solver;
/* storage: 0 f32, 1 f16 (x2^15, hash rounding), 2 bf16 (hash rounding) */
ow_solver *ow_create(uint32_t nx, uint32_t ny, uint32_t nz, float tau0, float u_in,
                     int les, int op, int walls, int storage,
                     const uint32_t *geometry, size_t geometry_len,
                     const uint32_t *boundary, size_t nboundary, int threads);
void ow_destroy(ow_solver *s);
/* free-slip faces (bit 0: y, bit 1: z; slip.h), 0 = the reference's periodic wrap */
void ow_set_lateral(ow_solver *s, int slip);
void ow_reset(ow_solver *s, float u_in_init);
/* one dispatch of stream_collide with the given inlet speed */
void ow_step(ow_solver *s, float u_in, int write_macro);
/* mean momentum exchange of both states (force.wgsl + reduce.wgsl), FP64 sum */
void ow_force(const ow_solver *s, double out[3]);
/* decoded populations g[i*cells+n] of the latest state */
void ow_populations(const ow_solver *s, float *out);
/* raw stored populations of the latest state (f32 bits or 16-bit codes) */
void ow_populations_raw(const ow_solver *s, void *out);
void ow_macros(const ow_solver *s, float *out);
/* overwrite the latest state's population i at cell n (decoded value) */
void ow_poke(ow_solver *s, uint32_t i, uint32_t n, float value);
void ow_params(const ow_solver *s, float out[4]); /* u_in, nu, cs_term, lambda */

/* ---- FP64 CpuSolver restatement ---- */
typedef struct oc_solver oc_solver;
/* op: 0 trt, 1 reg, 2 bgk; walls: 0 bb, 1 bouzidi.
 * flags: NULL (all fluid), cells entries, or packed geometry (2*cells+F).
 * init_state: NULL or cells*4 doubles (rho, ux, uy, uz) per cell. */
oc_solver *oc_create(uint32_t nx, uint32_t ny, uint32_t nz, double tau0, int op, int les,
                     const double body_force[3], int walls,
                     const uint32_t *flags, size_t flags_len,
                     const double eq_state[4], const double *init_state,
                     int threads, char *err, size_t errlen);
void oc_destroy(oc_solver *s);
/* free-slip faces as ow_set_lateral; rebuilds the pull sources from flags */
void oc_set_lateral(oc_solver *s, int slip, const uint32_t *flags, size_t flags_len, char *err, size_t errlen);
void oc_step(oc_solver *s);
void oc_macroscopic(oc_solver *s, uint32_t cell, double out[4]);
void oc_momentum_exchange(const oc_solver *s, double out[3]);
double *oc_populations(oc_solver *s);
size_t oc_cells(const oc_solver *s);
/* collision kernels used by collision.test.ts restatements */
void oc_equilibrium(double *target, double rho, const double u[3]);
void oc_moments(const double *g, double out[4]);
void oc_collide(double *g, const double *geq, double rho, double tau0, int op, int les,
                const double *force_terms);
int oc_collide_wall(double *g, const double *geq, double rho, const double u[3],
                    const int *wall_incoming, int nwall, double viscosity,
                    const double *force_terms);
double oc_friction_velocity(double speed, double viscosity);

/* ---- FP64 voxelizer + wall links ---- */
typedef struct {
  uint32_t solid_cells, frontal_cells, watertight, missed_links;
  double blockage;
  size_t geometry_len, nboundary;
} ov_stats;
/* Returns 0 on success, -1 on invalid input (message in err).  geometry and
 * boundary are malloc'd and must be released with ov_free. */
int ov_voxelize(const float *body, uint32_t ntri, const float *supports, uint32_t nsup,
                int has_supports, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on,
                int link_fractions, uint32_t **geometry, uint32_t **boundary,
                ov_stats *stats, char *err, size_t errlen);
int ov_build_wall_links(uint32_t *flags, const float *body, uint32_t ntri,
                        const float *supports, uint32_t nsup, int has_supports,
                        uint32_t nx, uint32_t ny, uint32_t nz, int floor_on, int measure,
                        uint32_t **geometry, uint32_t **boundary, ov_stats *stats);
void ov_free(void *p);
/* nearestLinkHit over triangle bins; returns 1 and writes t on a hit */
int ov_nearest_link_hit(const float *mesh, uint32_t ntri, uint32_t nx, uint32_t ny,
                        uint32_t nz, const double origin[3], const double dir[3], double *t);

/* ---- FP32 tracers ---- */
/* particles_update.wgsl: particles are 8 floats (pos.xyzw, prev.xyzw) */
void ot_particles_update(float *particles, uint32_t count, const float *macros,
                         const uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz,
                         uint32_t seed, float steps, const float cross_section[4],
                         const float fallback[2]);
uint32_t ot_hash(uint32_t v);
/* plate_smoke.wgsl: records vec4 (x, z, release, density) */
void ot_plate_smoke(float *smoke, uint32_t threads, uint32_t slots, uint32_t release,
                    int releasing, const float rake[4], uint32_t nx, uint32_t ny, uint32_t nz,
                    uint32_t plane, const float *macros, const uint32_t *flags,
                    const float *ports, uint32_t nports);
/* 3-D RK2 streaklines: records vec4 (x, y, z, density) + u32 release index */
void ot_streaks(float *puffs, uint32_t *release_of, uint32_t ry, uint32_t rz, uint32_t slots,
                uint32_t release, int releasing, const float rake[5], float h,
                uint32_t nx, uint32_t ny, uint32_t nz, const float *macros,
                const uint32_t *flags);

#ifdef __cplusplus
}
#endif
#endif
