/* dexmpm.h -- C ABI of libdexmpm.so, the GB300 (sm_103a) MLS-MPM substep of
 * DexDeform and its adjoint.
 *
 * Two groups of entry points:
 *
 *  1. Drop-in replacements for the reference's extern "C" kernel launchers
 *     (mpm/csrc/integrator.cu:1616-1985, bound by ctypes in mpm/types.py:130-290).
 *     Same names, argument order, AoS layouts (vec3 = 3 floats, mat3 = 9 floats
 *     row-major, quat = w,x,y,z) and dense x-major grids ((x*Gy + y)*Gz + z),
 *     same accumulate-into-gradient contract.  `ivec3 const &` arguments are
 *     passed as `const int *` (a C++ reference is a pointer at the ABI level).
 *     Differences: each returns an int status (0 = success) instead of void,
 *     and particles whose stencil leaves the grid are skipped and reported
 *     (DEXMPM_ERR_OUT_OF_GRID through dexmpm_get_error) instead of writing out
 *     of bounds.
 *
 *  2. The batched path (dexmpm_*): many environments of uneven particle counts
 *     advanced by one launch per phase, particles in SoA planes, grids in 4^3
 *     blocks with an active-block list.  Described by DexBatch below.
 *
 * All pointers are device pointers unless stated otherwise; `stream` is a
 * cudaStream_t (0 = legacy default stream).  Nothing here allocates device
 * memory: the caller owns every buffer.
 */
#ifndef DEXMPM_H
#define DEXMPM_H

#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef void *dexmpm_stream_t; /* cudaStream_t */

enum {
  DEXMPM_OK = 0,
  DEXMPM_ERR_ARG = 1,          /* bad argument (null pointer, bad size, bad layout) */
  DEXMPM_ERR_LAUNCH = 2,       /* CUDA launch error (cudaGetLastError after the launch) */
  DEXMPM_ERR_OUT_OF_GRID = 4,  /* device flag: a particle stencil left the grid; it was skipped */
  DEXMPM_ERR_TOO_MANY_BODIES = 8 /* more bodies per env than DEXMPM_MAX_BODIES */
};

#define DEXMPM_MAX_BODIES 32
#define DEXMPM_BLOCK 4 /* grid block edge, cells */

/* ===================================================================== 1 ==
 * Reference-compatible launchers.  Each cites the reference launcher it
 * replaces.  grid_lower must hold (0,0,0) (the reference never sets anything
 * else: mpm/simulator.py:16,386); it is read on the device as in the reference.
 */

/* integrator.cu:1627-1638 -- F_tmp = (I + dt C) F and its SVD. */
int compute_svd(float *F, float *C, float *newF, float *U, float *V, float *sig, float dt, int dim,
                dexmpm_stream_t stream);

/* integrator.cu:1640-1657 -- adjoint of compute_svd; accumulates F_grad, C_grad,
 * overwrites newF_grad with the full F_tmp gradient. */
int compute_svd_grad(float *F, float *C, float *U, float *V, float *sig, float *newF_grad, float *U_grad,
                     float *V_grad, float *sig_grad, float *F_grad, float *C_grad, float dt, int dim,
                     dexmpm_stream_t stream);

/* integrator.cu:1659-1690 -- von Mises projection and APIC/stress scatter. */
int p2g(float *particle_x, float *particle_v, float *particle_m, float *particle_vol, float *particle_F,
        float *particle_U, float *particle_sig, float *particle_V, float *particle_C,
        float *particle_mu_lam_yield, int *grid_lower, const int *grid_dim, float dx, float inv_dx, float dt,
        float *out_particle_F, float *out_grid_mv, float *out_grid_m, int dim, dexmpm_stream_t stream);

/* integrator.cu:1692-1742 -- adjoint of p2g. */
int p2g_grad(float *particle_x, float *particle_v, float *particle_m, float *particle_vol, float *particle_F,
             float *particle_U, float *particle_sig, float *particle_V, float *particle_C,
             float *particle_mu_lam_yield, int *grid_lower, const int *grid_dim, float dx, float inv_dx,
             float dt, float *out_particle_F, float *out_grid_mv, float *out_grid_m, float *particle_x_grad,
             float *particle_v_grad, float *particle_F_grad, float *particle_C_grad, float *particle_U_grad,
             float *particle_sig_grad, float *particle_V_grad, float *out_particle_F_grad,
             float *out_grid_v_grad, float *out_grid_m_grad, int dim, dexmpm_stream_t stream);

/* integrator.cu:1754-1779 -- gravity, sequential body contacts, walls and ground. */
int grid_op_v2(float *grid_m, float *grid_v_in, float *grid_body_v_in, int *grid_lower, float *gravity,
               float *body_pos, float *body_rot, float *next_body_pos, float *next_body_rot,
               float *body_type_friction_softness_round, float *body_args, float dx, float inv_dx, float dt,
               float ground_friction, float *out_grid_v, const int *grid_dim, int n_bodies,
               dexmpm_stream_t stream);

/* integrator.cu:1781-1819 -- adjoint of grid_op_v2. */
int grid_op_v2_grad(float *grid_m, float *grid_v_in, float *grid_body_v_in, int *grid_lower, float *gravity,
                    float *body_pos, float *body_rot, float *next_body_pos, float *next_body_rot,
                    float *body_type_friction_softness_round, float *body_args, float *grid_m_grad,
                    float *grid_v_in_grad, float *body_pos_grad, float *body_rot_grad, float *next_body_pos_grad,
                    float *next_body_rot_grad, float dx, float inv_dx, float dt, float ground_friction,
                    float *out_grid_v, float *out_grid_v_grad, const int *grid_dim, int n_bodies,
                    dexmpm_stream_t stream);

/* integrator.cu:1821-1835 -- APIC gather, advection and clamp. */
int g2p(float *particle_x, float *grid_v, int *grid_lower, float dx, float inv_dx, float dt,
        const int *grid_dim, float *out_particle_v, float ground_height, float *out_particle_C,
        float *out_particle_x, int dim, dexmpm_stream_t stream);

/* integrator.cu:1837-1861 -- adjoint of g2p. */
int g2p_grad(float *particle_x, float *grid_v, int *grid_lower, float dx, float inv_dx, float dt,
             const int *grid_dim, float *out_particle_v, float ground_height, float *out_particle_C,
             float *out_particle_x, int dim, float *particle_x_grad, float *grid_v_grad,
             float *out_particle_v_grad, float *out_particle_C_grad, float *out_particle_x_grad,
             dexmpm_stream_t stream);

/* integrator.cu:1935-1960 -- particle/body signed distances or their adjoint. */
int compute_dist(float *particle_x, float *body_pos, float *body_rot, float *body_type_friction_softness_round,
                 float *body_args, float *dist, int n_bodies, float *particle_x_grad, float *body_pos_grad,
                 float *body_rot_grad, float *dist_grad, int compute_grad, int dim, dexmpm_stream_t stream);

/* integrator.cu:1962-1984 -- per-object grid mass or its adjoint. */
int particle2mass(float *particle_x, float *particle_m, int *grid_lower, const int *grid_dim, float dx,
                  float inv_dx, float *out_grid_m, float *out_grid_m_grad, float *particle_x_grad,
                  int *particle_ids, int id, int compute_grad, int dim, dexmpm_stream_t stream);

/* Copy out and clear the error word shared by the launchers above (host
 * pointer out; synchronous).  No counterpart in the reference, which has no
 * error reporting (mpm/csrc/common.h:20-34). */
int dexmpm_abi_get_error(int32_t *out);

/* Renderer (mpm/renderer.py:88-169).  All pointers are device pointers.
 *
 * integrator.cu:1911-1933 -- bake a particle volume: splat every particle
 * into the (2 bake_size)^3 voxels around it with a 64-bit atomicMin of
 * (quantised distance << 24 | rgb) into `volume` (filled with (1 << 33) - 1 by
 * the caller), unpack distance / 255 into sdf and rgb / 255 into color
 * (float[3] per voxel), then two 3^3 box filters of sdf (border voxels 1;
 * sdf_tmp is scratch).  Voxel (i, j, k) of the x-major grid_dim lies at
 * bbox_min + (i, j, k) / inv_dx.  Bit-identical to the reference. */
int particle_sdf(long long *volume, float *particle_x, int *particle_color, float *bbox_min, float *bbox_max,
                 int bake_size, const int *grid_dim, float inv_dx, float *sdf, float *color, float *sdf_tmp,
                 int n_particles, dexmpm_stream_t stream);

/* integrator.cu:1862-1905 -- path-traced image (image_dim = rows, cols) of the
 * ground plane, n_bodies (<= 64) SDF bodies and, when visualize_shape, the
 * baked volume's sdf_threshold level set: spp jittered samples per pixel,
 * max_ray_depth diffuse bounces with a shadow ray towards light_direction.
 * color_buffer receives float[3] per pixel (vignette, exposure 1.5, sqrt),
 * depth_buffer the distance of the first hit (1e9 for sky), averaged over
 * the samples.  Random numbers: SplitMix64 of (seed, pixel, draw index) in
 * (0, 1], drawn in the reference's order, instead of curand XORWOW states
 * (which the reference allocates on every call). */
int render(float *sdf_volume, float *box_min, float *box_max, float *color_volume, float *body_pos, float *body_rot,
           float *body_type_friction_softness_round, float *body_args, float *camera_rot, float *camera_pos,
           float *camera_intrinsic, float *color_buffer, float *depth_buffer, float sdf_threshold, const int *grid_dim,
           int n_bodies, bool visualize_shape, const int *image_dim, int max_ray_depth, int spp, float ground_height,
           int seed, float *light_direction, dexmpm_stream_t stream);

/* ===================================================================== 2 ==
 * Batched path.
 *
 * Particle state slot: 24 float planes of n_particles each, plane-major:
 *   x 0-2, v 3-5, F 6-14 (row-major), C 15-23.  Gradient slots use the same layout.
 * Material: mass[n], vol[n], mu_lam_yield[3][n] (planes mu, lambda, yield).
 * Grids: every env owns gx*gy*gz cells (dims multiples of 4) stored as 4^3
 *   blocks; block b of the whole batch holds cells [64b, 64b+64), cell
 *   (x,y,z) of env e is block blk_off + ((x>>2)*(gy/4) + (y>>2))*(gz/4) + (z>>2),
 *   slot ((x&3)*16 + (y&3)*4 + (z&3)).  Cell values are float4.
 * Grid slots: `n_slots` copies of
 *     grid   (m v.x, m v.y, m v.z, m) after P2G
 *     vout   (v.x, v.y, v.z, c) after the grid update; c holds, as uint32
 *            bits, the env's bodies whose contact changed the node (bit b:
 *            body b), which the grid adjoint replays
 *   with a block flag array, an active-block list and its count per slot.
 *   P2G into slot k appends the blocks its stencils touch to slot k's list.
 *   Forward substeps alternate two slots; each grid update clears the slot of
 *   the previous substep (clear_slot).  The adjoint of a substep reads the
 *   slot its forward left behind and clears it, so recomputed substeps can
 *   keep one slot each until their adjoint runs.  No per-substep memset.
 * Gradient grids (one each): vout_grad dL/dv_out, in_grad (dL/d(mv), dL/dm);
 *   the grid adjoint zeroes vout_grad after reading it and writes in_grad for
 *   every cell of its blocks.
 * Alignment: the kernels read and write grid, vout, vout_grad, in_grad,
 *   body_shape and the pose arrays as float4, so each must start on a 16-byte
 *   boundary (cudaMalloc'd buffers and whole rows of them do); the launchers
 *   return DEXMPM_ERR_ARG for one that does not.  State, material, tape and
 *   pose-gradient arrays need only float alignment.
 * Poses: [n_bodies][8] floats per substep boundary: p.x p.y p.z 0 q.w q.x q.y q.z.
 * Body shapes: [n_bodies][8]: type friction softness round, args w x y z.
 * Body-pose gradients: [n_bodies][8] in the pose layout, accumulated.
 */
typedef struct {
  int32_t p_off, n, blk_off, body_off; /* first particle, count, first grid block, first body */
  int32_t gx, gy, gz, n_bodies;        /* grid dims (multiples of 4), bodies */
  float dx, inv_dx, dt, ground_friction;
  float gravity[3];
  float ground_height; /* cells; the particle clamp is [gh*dx, (G-3)*dx] */
} DexEnv;              /* 64 bytes */

/* DexBatch.flags bits */
#define DEXMPM_FLAG_EXACT_CAPSULE_GRAD 1 /* true capsule-normal derivative in the grid adjoint; the
                                            reference drops it (mpm/csrc/shape.h:138-148) */

typedef struct {
  int32_t n_envs, n_particles, n_tiles, n_blocks;
  int32_t n_bodies, tile_size, grid_ctas, flags; /* flags: DEXMPM_FLAG_* */
  int32_t n_slots, pad0, pad1, pad2;
  const DexEnv *envs;         /* [n_envs] */
  const int32_t *tiles;       /* [n_tiles][2]: env, first particle within the env */
  const int32_t *block_env;   /* [n_blocks]: owning env */
  const float *mass;          /* [n_particles] */
  const float *vol;           /* [n_particles] */
  const float *mu_lam_yield;  /* [3][n_particles] */
  float *grid;                /* [n_slots][n_blocks*64] float4 */
  float *vout;                /* [n_slots][n_blocks*64] float4 */
  float *vout_grad;           /* [n_blocks*64] float4, nullable without gradients */
  float *in_grad;             /* [n_blocks*64] float4, nullable without gradients */
  uint32_t *block_flag;       /* [n_slots][n_blocks] */
  int32_t *block_list;        /* [n_slots][n_blocks] */
  int32_t *block_count;       /* [n_slots] */
  uint32_t *done_counter;     /* [1] */
  const float *body_shape;    /* [n_bodies][8] */
  int32_t *error;             /* [1] sticky DEXMPM_ERR_* bits */
  const int32_t *block_xyz;   /* [n_blocks]: the block's coordinates in its env's grid of 4^3
                                 blocks, bx << 20 | by << 10 | bz (up to 1,023 blocks per axis) */
} DexBatch;

/* Zero every grid slot, flag, list count and the error word.  Call once after
 * allocation -- the slot protocol keeps them clean afterwards. */
int dexmpm_reset(const DexBatch *b, dexmpm_stream_t stream);

/* P2G into grid slot `slot`: SVD, von Mises, stress, APIC scatter of state
 * slot s; appends the touched blocks to the slot's list.  next_s (nullable)
 * receives the projected F (its 9 F planes).  tape (nullable): DEXMPM_TAPE_PLANES
 * planes of n_particles floats that receive each particle's SVD of F_tmp and
 * stress (U 0-8, V 9-17, sigma 18-20, sigma - 1 21-23, P 24-32 before the
 * -dt vol 4 inv_dx^2 scale) for the adjoint of this substep. */
#define DEXMPM_TAPE_PLANES 33
int dexmpm_p2g(const DexBatch *b, int slot, const float *s, float *next_s, float *tape, dexmpm_stream_t stream);

/* Grid update on the active blocks of `slot`, with body poses at the substep
 * start (pose) and end (next_pose); then clears grid slot clear_slot (< 0: none). */
int dexmpm_grid_op(const DexBatch *b, int slot, int clear_slot, const float *pose, const float *next_pose,
                   dexmpm_stream_t stream);

/* G2P from grid slot `slot`: x, v, C of next_s from s. */
int dexmpm_g2p(const DexBatch *b, int slot, const float *s, float *next_s, dexmpm_stream_t stream);

/* G2P of substep t from grid slot slot_g fused with the P2G of substep t + 1
 * into slot slot_s: x, v, C of state t + 1 to next_s from x of state s; then,
 * with the F of state t + 1 already in next_s (written by the P2G of substep
 * t), that state's SVD, stress and scatter, its projected F to s2's F planes
 * and its tape (nullable).  s2 may be s (only x is read from s, only F is
 * written to s2).  Same results as dexmpm_g2p(slot_g) + dexmpm_p2g(slot_s)
 * without reloading state t + 1 or a second launch. */
int dexmpm_g2p2g(const DexBatch *b, int slot_g, int slot_s, const float *s, float *next_s, float *s2, float *tape,
                 dexmpm_stream_t stream);

/* One forward substep: dexmpm_p2g + dexmpm_grid_op + dexmpm_g2p. */
int dexmpm_substep(const DexBatch *b, int slot, int clear_slot, const float *s, float *next_s, const float *pose,
                   const float *next_pose, float *tape, dexmpm_stream_t stream);

/* Adjoint of the substep whose forward (p2g + grid_op) filled grid slot
 * `slot` from state s.  next_s is the state after the substep (its v sets the
 * clamp mask), g_next the gradient of next_s, g the gradient of s
 * (overwritten).  Body-pose gradients are added to bgrad / next_bgrad.  The
 * slot is cleared for reuse.  tape (nullable): the tape the forward P2G of this
 * substep wrote; without it the adjoint recomputes the SVD and return mapping. */
int dexmpm_substep_grad(const DexBatch *b, int slot, const float *s, const float *next_s, const float *g_next,
                        float *g, const float *pose, const float *next_pose, float *bgrad, float *next_bgrad,
                        const float *tape, dexmpm_stream_t stream);

/* The three kernels of dexmpm_substep_grad, callable one by one: G2P adjoint
 * (writes the x gradient of s, scatters dL/dv_out), grid-update adjoint
 * (dL/d(mv), dL/dm, body-pose gradients; clears the slot), P2G + SVD adjoint
 * (completes the gradient of s). */
int dexmpm_g2p_grad(const DexBatch *b, int slot, const float *s, const float *next_s, const float *g_next,
                    float *g, dexmpm_stream_t stream);
int dexmpm_grid_op_grad(const DexBatch *b, int slot, const float *pose, const float *next_pose, float *bgrad,
                        float *next_bgrad, dexmpm_stream_t stream);
int dexmpm_p2g_grad(const DexBatch *b, int slot, const float *s, const float *g_next, float *g, const float *tape,
                    dexmpm_stream_t stream);

/* P2G adjoint of substep t (grid slot `slot`, after its grid-update adjoint)
 * fused with the G2P adjoint of substep t - 1 (grid slot prev_slot): s is
 * state t, prev_s state t - 1, g_next the gradient of state t + 1 (its F is
 * read), g the gradient of state t (its x holds the G2P adjoint's part; its F
 * is written), g_prev the gradient of state t - 1 (its x is written; may be
 * g_next).  The x, v, C gradients of state t pass between the two adjoints in
 * registers and are not stored.  Same results as dexmpm_p2g_grad(slot) +
 * dexmpm_g2p_grad(prev_slot) apart from those three stores, in one launch. */
int dexmpm_p2g_g2p_grad(const DexBatch *b, int slot, int prev_slot, const float *s, const float *prev_s,
                        const float *g_next, float *g, float *g_prev, const float *tape, dexmpm_stream_t stream);

/* Clear grid slots [first, last) whose adjoint will not run (their listed
 * blocks, flags and list counts), e.g. substeps kept for an adjoint that was
 * not taken.  No counterpart in the reference. */
int dexmpm_clear_slots(const DexBatch *b, int first, int last, dexmpm_stream_t stream);

/* One forward substep (P2G, grid update, G2P) of ONE environment that
 * allocates no device memory: for callers that cannot call cudaMalloc, such
 * as a host application whose own pool allocator owns the device memory, or
 * a real-time loop that must not block on or fail in an allocation.  No
 * counterpart in the reference.
 *   env:    HOST pointer; p_off = blk_off = body_off = 0; grid dims multiples
 *           of 4 with gx*gy*gz <= 262144 (64^3); n <= 1048576; n_bodies <= 32.
 *   s, next_s: state slots of 24 planes of env->n floats (layout above).
 *   mass, vol [n], mu_lam_yield [3][n]; body_shape, pose, next_pose [n_bodies][8].
 *   error:  device int32, required; DEXMPM_ERR_OUT_OF_GRID is OR-ed in when
 *           a particle stencil leaves the grid (that particle is skipped).
 *           It is not cleared by the call.
 * Grids, active-block lists and counters live in one fixed device array of
 * this library (8.5 MB, held by every GPU that loads it until exit), shared
 * by all calls: each call clears what must start at zero, and calls that
 * overlap on the GPU race on it.  Each call looks up the array's device
 * address; the first call on a device also loads the library's device code
 * there, so make that first call before any stream capture.
 * Returns DEXMPM_ERR_ARG for sizes beyond the limits, a null pointer among
 * the required ones, and dx, inv_dx or dt that are not positive and finite or
 * with dx * inv_dx != 1. */
int dexmpm_substep_noalloc(const DexEnv *env, const float *s, float *next_s, const float *mass, const float *vol,
                           const float *mu_lam_yield, const float *body_shape, const float *pose,
                           const float *next_pose, int32_t *error, dexmpm_stream_t stream);

/* ------------------------------------------------------------------------
 * Particle order.  The scatters pre-reduce a warp's contributions per stencil
 * base, which pays when particles that are close in space are close in
 * memory.  dexmpm_sort re-orders every env's particles (within the env's
 * range) by the 4^3 block of their stencil base cell, then by the cell
 * within the block, then by their previous index: a counting sort in one
 * launch per phase for all envs.  No counterpart in the reference, which
 * scatters in the caller's order (mpm/csrc/integrator.cu:312-394).
 *
 * DexSortWork: caller-owned device scratch, all zero before the first sort
 * (each sort leaves cell_count, block_total, block_flag and counters zero).
 * cell_count and cell_start are accessed as int2 (8-byte aligned starts),
 * block_total as int4 (16-byte aligned); otherwise DEXMPM_ERR_ARG. */
#define DEXMPM_STATE_PLANES 24
#define DEXMPM_SORT_CHUNK 4096 /* block totals per scan CTA */
#define DEXMPM_SORT_PARTIALS(n_blocks) (((n_blocks) + DEXMPM_SORT_CHUNK - 1) / DEXMPM_SORT_CHUNK)
typedef struct {
  int32_t *cell_count;  /* [n_blocks * 64] */
  int32_t *cell_start;  /* [n_blocks * 64] */
  int32_t *block_total; /* [n_blocks] */
  int32_t *block_base;  /* [n_blocks] */
  uint32_t *block_flag; /* [n_blocks] */
  int32_t *block_list;  /* [n_blocks] */
  int32_t *rank;        /* [n_particles] */
  int32_t *key;         /* [n_particles] */
  int32_t *partial;     /* [DEXMPM_SORT_PARTIALS(n_blocks)] */
  int32_t *counters;    /* [4] */
} DexSortWork;

/* Sort the particles of state slot s: perm[i] = the index in s of the
 * particle that goes to index i (entries of the padding beyond the envs'
 * particles are left as they are: initialise perm to the identity once), and
 * sorted_s = s gathered by perm (24 planes).  s and sorted_s must differ.  At
 * most 4,194,304 grid blocks. */
int dexmpm_sort(const DexBatch *b, const DexSortWork *w, const float *s, float *sorted_s, int32_t *perm,
                dexmpm_stream_t stream);

/* Apply a permutation to `planes` planes of n 32-bit words (floats or
 * int32): inverse = 0 gathers dst[q][i] = src[q][perm[i]] (into the sorted
 * order), inverse = 1 scatters dst[q][perm[i]] = src[q][i] (back to the
 * previous order, e.g. gradients).  src and dst must differ. */
int dexmpm_permute(const int32_t *perm, const void *src, void *dst, int n, int planes, int inverse,
                   dexmpm_stream_t stream);

/* One block of a segmented plane copy: `count` consecutive floats in each
 * of `planes` planes, at `other` (plane q at other + q * other_stride) and
 * at column `offset` of the shared buffer (plane q at buf + q * buf_stride +
 * offset). */
typedef struct {
  float *other;
  int32_t other_stride, offset, count, pad;
} DexSegment; /* 24 bytes */

#define DEXMPM_SEGMENTS_GATHER 0      /* buf <- other */
#define DEXMPM_SEGMENTS_SCATTER 1     /* other <- buf */
#define DEXMPM_SEGMENTS_SCATTER_ADD 2 /* other += buf */

/* Many blocks of planes between their own buffers and one shared buffer in
 * one launch per DEXMPM_SEGMENTS_PER_LAUNCH segments (the serving loop
 * gathers its requests' states, gradients and poses into an engine and
 * scatters the results back this way).  seg is a HOST array of n segments,
 * passed to the kernel in its launch parameters (no copy to the device and
 * no synchronisation; the array may be reused as soon as the call returns);
 * every segment copies `planes` planes.  The segments' columns in buf must
 * not overlap for a gather, nor their `other` blocks for a scatter. */
#define DEXMPM_SEGMENTS_PER_LAUNCH 512
int dexmpm_copy_segments(const DexSegment *seg, int n, int planes, float *buf, int buf_stride, int mode,
                         int max_count, dexmpm_stream_t stream);

/* Copy out and clear the device error word (host pointer out). */
int dexmpm_get_error(const DexBatch *b, int32_t *out, dexmpm_stream_t stream);

/* Library version string (host). */
const char *dexmpm_version(void);

#ifdef __cplusplus
}
#endif
#endif
