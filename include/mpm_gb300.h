/*
 * mpm_gb300.h -- C ABI of the GB300 (sm_103a) differentiable MLS-MPM substep.
 *
 * Drop-in boundary for the hot path of DiffSkill's plb/engine: the Taichi
 * kernels of plb/engine/mpm_simulator.py (p2g, grid_op, g2p, compute_grid_m,
 * their autodiff twins) and the tool kinematics of
 * plb/engine/primitive/primive_base.py.  Host code (Python, ctypes) keeps the
 * reference's API and owns all state buffers; this library receives raw
 * device pointers and sizes, launches on the caller's CUDA stream, and never
 * frees caller memory.  The only memory it owns is the per-handle grid
 * scratch allocated by mpm_create and freed by mpm_destroy.
 *
 * Layouts (all device pointers, "real" = float or double per precision):
 *   particle state of one frame: real[24][ld], component-major (SoA):
 *       rows 0-2 x, 3-5 v, 6-14 C (row-major 3x3), 15-23 F (row-major 3x3);
 *       particles of scene s occupy columns [scene_offsets[s], scene_offsets[s+1]).
 *   grid (density, target): real[n_scenes][n_grid^3], node (i,j,k) at
 *       (i*n + j)*n + k, the C order of the reference's 64^3 / 128^3 fields.
 *   tool pose of one frame: double[n_tools][8] = pos[3], rot[4] (w,x,y,z), gap.
 *   tool velocity of one substep: double[n_tools][8] = v[3], w[3], gap_vel, 0.
 *   action of one step: double[n_tools][8] (first action_dim entries used).
 *
 * Every entry point returns 0 (MPM_OK) or an MPM_E_* code; mpm_last_error
 * gives the message.  Kernels never trap: numerical faults and particles whose
 * stencil leaves the grid set bits of a sticky device status word that
 * mpm_status reads back.
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPM_ABI_VERSION 6

/* return codes */
#define MPM_OK 0
#define MPM_E_INVALID 1   /* bad argument, size or pointer */
#define MPM_E_CUDA 2      /* a CUDA runtime call failed */
#define MPM_E_NOMEM 3     /* scratch allocation failed */

/* precision modes (SIMULATOR.dtype of plb/config/default_config.py:15) */
#define MPM_PREC_FP32 0       /* FP32 state/grid/SVD, FP64 reductions */
#define MPM_PREC_FP32_SVD64 1 /* FP32 state/grid, FP64 SVD + return map + adjoint */
#define MPM_PREC_FP64 2       /* all FP64: the plain reference method */

/* tool types (plb/engine/primitive/primitives.py) */
#define MPM_TOOL_SPHERE 0  /* Sphere   primitives.py:23-40 */
#define MPM_TOOL_CAPSULE 1 /* Capsule  primitives.py:43-91 */
#define MPM_TOOL_BOX 2     /* Box      primitives.py:359-425 */
#define MPM_TOOL_KNIFE 3   /* Knife = Prism ∩ Box, primitives.py:700-815 */
#define MPM_TOOL_GRIPPER 4 /* Gripper  primitives.py:428-573 */
#define MPM_TOOL_ROLLINGPIN 5    /* RollingPin    primitives.py:101-117 (Capsule shape) */
#define MPM_TOOL_ROLLINGPINEXT 6 /* RollingPinExt primitives.py:120-135 (Capsule shape) */
#define MPM_TOOL_CHOPSTICKS 7    /* Chopsticks    primitives.py:218-290 */
#define MPM_TOOL_CYLINDER 8      /* Cylinder      primitives.py:293-326 */
#define MPM_TOOL_TORUS 9         /* Torus         primitives.py:329-356 */
#define MPM_TOOL_GRIPPER2 10     /* Gripper2      primitives.py:576-697 (Capsule fingers) */

/* status bits (sticky; cleared by mpm_status with clear=1) */
#define MPM_STATUS_OUT_OF_GRID 1u /* a particle stencil left the grid; it was skipped */
#define MPM_STATUS_NONFINITE 2u   /* a NaN/Inf velocity or deformation was produced */
#define MPM_STATUS_RENDER_BOX 4u  /* mpm_render_bake: the particles' box exceeds the render volume */

/* Simulator constants: MPMSimulator.__init__ (mpm_simulator.py:8-67). */
typedef struct MpmParams {
  int32_t abi_version; /* MPM_ABI_VERSION */
  int32_t precision;   /* MPM_PREC_* */
  int32_t n_grid;      /* nodes per axis (64 or 128 in the workloads) */
  int32_t n_scenes;    /* independent scenes batched in one launch */
  int64_t n_particles; /* total over scenes */
  int64_t ld;          /* leading dimension of state rows, >= n_particles */
  double dx, inv_dx, dt, p_vol, p_mass;
  double mu, lam, yield_stress; /* Lame parameters and von Mises yield */
  double gravity[3];            /* multiplied by 30 in grid_op (mpm_simulator.py:235) */
  double ground_friction;
  double lower_bound;
} MpmParams;

/* One rigid tool: Primitive cfg (primive_base.py:313-329) + shape fields. */
typedef struct MpmToolDesc {
  int32_t type;       /* MPM_TOOL_* */
  int32_t action_dim; /* cfg.action.dim */
  int32_t scene;      /* owning scene; tools must be sorted by scene */
  /* bit j set: collision_group[j] > 0, i.e. this tool is projected out of
   * the scene's tool j (a Box) after every forward-kinematics step
   * (mpm_simulator.py:69-80, 287-305); j counts the scene's tools from 0 */
  int32_t collision_mask;
  double friction, softness;
  double radius;        /* Sphere */
  double cap_h, cap_r;  /* h, r: Capsule, RollingPin(Ext), Chopsticks, Gripper2 fingers;
                           Cylinder: h = radial extent, r = half height (primitives.py:300-304) */
  double size[3];       /* Box / Knife box / Gripper finger half extents */
  double prism_h[2];    /* Knife prism h */
  double prot[4];       /* Knife prism rotation */
  double min_gap, max_gap;
  double lower[3], upper[3];
  double action_scale[7];
  double torus[2];      /* Torus tx, ty */
} MpmToolDesc;

/* Grid store (caller-owned device buffers): the forward grids of a substep,
 * i.e. its active 4x4x4-node blocks of the p2g grid and of the grid_op
 * output, kept so the adjoint substep restores both instead of recomputing
 * p2g and grid_op.  Slots are filled by a device-side bump
 * allocator; a substep that does not fit gets slot_start = -1 and its adjoint
 * recomputes the grid, so results never depend on the capacity.  Zero *bump
 * (and set slot_start to -1) before reusing slots. */
typedef struct MpmGridStore {
  void* blocks;                 /* real[capacity][2][64][4]: p2g grid block, grid_op output block */
  int32_t* block_ids;           /* [capacity] global block id of each stored block */
  int64_t* slot_start;          /* [n_slots] first stored block of the slot, -1 = not stored */
  int32_t* slot_count;          /* [n_slots] */
  unsigned long long* bump;     /* [1] blocks handed out so far */
  int64_t capacity;             /* blocks */
  int32_t n_slots;
  int32_t reserved;
} MpmGridStore;

/* Launch shapes of the substep kernels (no counterpart in the reference,
 * whose launch shapes are Taichi's).  A field of 0 keeps the default.  The
 * FP32 particle kernels are compiled for several CTAs-per-SM targets (each a
 * register budget: 65536 / (128 * CTAs) registers per thread); the grid
 * kernels stride over the active blocks with grid_ctas_per_sm * SMs CTAs.
 * diffskill_gb300/autotune.py times the candidates and picks per workload. */
typedef struct MpmTuning {
  int32_t p2g_ctas;          /* FP32 p2g: 6, 7 (default) or 8 CTAs of 128 threads per SM */
  int32_t g2p_adj_ctas;      /* FP32 g2p.grad: 5, 6 (default), 7 or 8 */
  int32_t p2g_adj_ctas;      /* FP32 p2g.grad: 4, 5 (default) or 6 */
  int32_t grid_ctas_per_sm;  /* grid_op / grid_op.grad: 2 .. 64 (default 16) */
  int32_t g2p_ctas;          /* FP32 g2p: 8 (default: the compiler's 64 registers), 10 or 12 */
  int32_t grid_op_adj_ctas;  /* FP32 grid_op.grad, CTAs of 64 threads: 6 (default: the compiler's choice),
                                12 or 16 */
} MpmTuning;

typedef struct MpmHandle MpmHandle;

const char* mpm_version(void);

/* MPMSimulator.__init__ + initialize (mpm_simulator.py:8-97).
 * scene_offsets: host int64[n_scenes+1], particle column ranges per scene.
 * Allocates the grid scratch (4 grids of n_scenes*n_grid^3 nodes). */
int mpm_create(const MpmParams* params, const int64_t* scene_offsets, MpmHandle** out);
int mpm_destroy(MpmHandle* h);

/* Primitives.__init__/initialize (primitives.py:820-897): tool table.
 * tools: host array, sorted by scene; copied to the device. */
int mpm_set_tools(MpmHandle* h, const MpmToolDesc* tools, int32_t n_tools);

/* The random numbers of the tool-tool collision projection: points[c][k][3]
 * for the c-th collision pair of a scene (c < n_pairs) and k < 600, drawn as
 * the reference draws rand_num (np.random.seed(42); uniform(-1.5, 1.5,
 * (n_pairs, 600, 3)), mpm_simulator.py:89-96).  Host array, copied.  Needed
 * when any tool has a collision_mask. */
int mpm_set_collision_points(MpmHandle* h, const double* points, int32_t n_pairs);
/* Number of collision pairs over all scenes (rows of a coll record). */
int mpm_collision_pairs(MpmHandle* h);

/* Primitive.set_action + set_velocity + forward_kinematics for the n_sub
 * substeps of one action (primive_base.py:152-156, 246-274; per-type
 * kinematics of primitives.py: RollingPin 104-117, RollingPinExt 122-135,
 * Chopsticks 231-245, Gripper 457-469, Gripper2 589-601), each substep
 * followed by the tool-tool collision projection of MPMSimulator.substep
 * (mpm_simulator.py:287-305, 316-319): every pair (i, j) takes the first of
 * 600 points of box j's surface with the most negative SDF of tool i (none
 * if no SDF is below 0) and moves tool i by normalized(normal) * SDF there.
 * action: double[n_tools][8] (clipped by the caller); vel:
 * double[n_sub][n_tools][8] written; pose: double[n_sub+1][n_tools][8] with
 * frame 0 given, frames 1..n_sub written; coll: double[n_sub][n_pairs][4]
 * written (chosen point index or -1, then the point), NULL if there are no
 * collision pairs.  One launch; the 600 points are evaluated in parallel and
 * the lowest index wins ties. */
int mpm_tools_action(MpmHandle* h, const double* action, double* vel, double* pose, double* coll, int32_t n_sub,
                     void* stream);
/* Adjoint: set_velocity.grad + forward_kinematics.grad (function.py:180-182)
 * and, per substep before them, apply_collision_projection.grad and
 * set_surface_points.grad (mpm_simulator.py:337-339), evaluated like the
 * reference's autodiff at the stored (projected) poses and stored points.
 * g_pose: double[n_sub+1][n_tools][8] accumulated gradients of every frame on
 * entry; on exit g_pose[0] also holds what reaches frame 0.  g_action:
 * double[n_tools][8] accumulated. */
int mpm_tools_action_bwd(MpmHandle* h, const double* vel, const double* pose, const double* coll, double* g_pose,
                         double* g_action, int32_t n_sub, void* stream);

/* One substep (MPMSimulator.substep, mpm_simulator.py:307-323, without the
 * forward_kinematics that mpm_tools_action already ran): clear_grid,
 * compute_F_tmp, svd, p2g, grid_op, g2p.  state_f -> state_f1 (distinct
 * buffers).  pose_f, pose_f1: double[n_tools][8] of frames f and f+1. */
int mpm_substep_fwd(MpmHandle* h, const void* state_f, void* state_f1, const double* pose_f, const double* pose_f1,
                    void* stream);

/* Adjoint of one substep (MPMSimulator.substep_grad, mpm_simulator.py:325-345:
 * recompute grid, g2p.grad, grid_op.grad, p2g.grad, svd_grad,
 * compute_F_tmp.grad).  g_state_f1 -> g_state_f (overwritten).
 * state_f1 (may be NULL): frame f+1 as the forward produced it; its v rows
 * replace a second grid gather in g2p.grad.
 * g_pose_f, g_pose_f1: double[n_tools][8], accumulated. */
int mpm_substep_bwd(MpmHandle* h, const void* state_f, const void* state_f1, const void* g_state_f1,
                    void* g_state_f, const double* pose_f, const double* pose_f1, double* g_pose_f,
                    double* g_pose_f1, void* stream);

/* Chained forward substeps (on = 1; off by default).  While on, each forward
 * substep's g2p also flags the grid blocks of its output frame, and a forward
 * substep whose input frame is the previous forward substep's output skips
 * its own marking pass.  Contract: between two such substeps the frame is
 * not modified, except by a permutation of the particles within their scene
 * columns (the re-sort), which leaves the set of blocks unchanged.  Any
 * adjoint substep ends the chain.  No counterpart in the reference. */
int mpm_set_chained(MpmHandle* h, int32_t on);

/* Pipelined adjoint substeps (on = 1; off by default).  While on, an
 * adjoint substep (mpm_substep_bwd / mpm_substep_bwd_store) that follows
 * another on the same stream runs its grid preparation (active blocks, pose
 * table, forward grids restored from the store or recomputed) on an internal
 * stream, beside the previous substep's p2g.grad; its g2p.grad waits for both.
 * Contract: between two such calls the caller's stream runs nothing that
 * writes the handle's grids or pose table (no forward substep; a frame
 * gradient permutation, the losses' adjoints and the tool kinematics adjoint
 * are fine).  A forward substep, a change of stream or turning it off or on
 * again ends the overlap.  The internal stream and its two events belong to
 * the handle (created by mpm_create).  No counterpart in the reference. */
int mpm_set_pipelined_adjoint(MpmHandle* h, int32_t on);

/* Sets the launch shapes of the handle's later substeps (MpmTuning; a value
 * outside a field's candidates returns MPM_E_INVALID and changes nothing).
 * No counterpart in the reference. */
int mpm_set_tuning(MpmHandle* h, const MpmTuning* tuning);
/* Reads the handle's launch shapes, defaults filled in. */
int mpm_get_tuning(MpmHandle* h, MpmTuning* tuning);

/* mpm_substep_fwd that also keeps the substep's forward grids in store slot
 * `slot` (no counterpart in the reference, whose substep_grad always
 * recomputes the grid, mpm_simulator.py:327-333). */
int mpm_substep_fwd_store(MpmHandle* h, const void* state_f, void* state_f1, const double* pose_f,
                          const double* pose_f1, const MpmGridStore* store, int32_t slot, void* stream);
/* mpm_substep_bwd that restores the forward grids (p2g grid and grid_op
 * output) from store slot `slot` when they were stored, and recomputes them
 * otherwise. */
int mpm_substep_bwd_store(MpmHandle* h, const void* state_f, const void* state_f1, const void* g_state_f1,
                          void* g_state_f, const double* pose_f, const double* pose_f1, double* g_pose_f,
                          double* g_pose_f1, const MpmGridStore* store, int32_t slot, void* stream);

/* Particle re-sort (no counterpart in the reference: Taichi scatters into its
 * dense fields in launch order, mpm_simulator.py:199-225).  Sorts the
 * particles of frame src by (scene, 4^3 grid block, cell), stably, and
 * writes the sorted frame (all 24 rows) to dst: dst[:, i] = src[:, perm[i]].
 * Particles stay inside their scene, so losses and action gradients do not
 * change.  perm: int32[n_particles] (device, 4-byte aligned) receives the
 * permutation.  src and dst must not overlap.  Needs n_particles < 2^31 and
 * n_scenes * n_grid^3 < 2^32 (MPM_E_INVALID otherwise).  The block flags a
 * chained forward substep set for src are kept for dst.  No allocation;
 * capturable. */
int mpm_sort_frame(MpmHandle* h, const void* src, void* dst, int32_t* perm, void* stream);
/* Adjoint of mpm_sort_frame for a frame gradient: g_dst[:, perm[i]] =
 * g_src[:, i] (all 24 rows).  g_src and g_dst must not overlap. */
int mpm_unsort_frame(MpmHandle* h, const void* g_src, void* g_dst, const int32_t* perm, void* stream);

/* compute_grid_m_kernel on a cleared grid (mpm_simulator.py:456-471).
 * grid_m: real[n_scenes][n_grid^3] written. */
int mpm_grid_mass(MpmHandle* h, const void* state, void* grid_m, void* stream);
/* compute_grid_m_kernel.grad (function.py:147-152): accumulates the x rows
 * of g_state from g_grid_m (real[n_scenes][n_grid^3]). */
int mpm_grid_mass_bwd(MpmHandle* h, const void* state, const void* g_grid_m, void* g_state, void* stream);

/* compute_density_loss_kernel (loss.py:172-175) per scene, FP64 reduction:
 * loss[s] = weight * sum_I |grid_m - target|  (double[n_scenes], overwritten);
 * if g_grid_m is not NULL it receives weight * sgn(grid_m - target). */
int mpm_density_l1(MpmHandle* h, const void* grid_m, const void* target, double weight, double* loss,
                   void* g_grid_m, void* stream);

/* Soft contact distance (loss.py:143-162) of every tool of every scene at one
 * frame: min_dist[t] = sum_i d_i w_i / sum_i w_i, d_i = max(sdf_t(x_i), 0),
 * w_i = 1/(1+1e4 d_i^2), over the particles of the tool's scene, in FP64.
 * Tools with action_dim 0 are skipped (Loss keeps movable tools only,
 * loss.py:21-25).  sums: double[n_tools][2] = (sum w, sum d w) written;
 * min_dist: double[n_tools] written. */
int mpm_soft_contact(MpmHandle* h, const void* state, const double* pose, double* sums, double* min_dist,
                     void* stream);
/* Adjoint given the forward sums and g_min_dist (double[n_tools]):
 * accumulates the x rows of g_state and g_pose (double[n_tools][8]). */
int mpm_soft_contact_bwd(MpmHandle* h, const void* state, const double* pose, const double* sums,
                         const double* g_min_dist, void* g_state, double* g_pose, void* stream);

/* update_target (loss.py:129-134): update_target_sdf (loss.py:105-124)
 * iterated n_iters times from a copy filled with inf = 1000 (the reference
 * runs 2*n_grid iterations).  A node with target density > 1e-4 gets sdf 0
 * and itself as nearest point; any other node the first strict minimum over
 * the offsets (-3..2)^3 \ {0}, in the reference's loop order, of
 * sqrt(|I*dx - nearest_copy[v]|^2 + 1e-8) over neighbours with sdf_copy < inf,
 * else inf.  target_density: real[n_scenes][n_grid^3]; target_sdf:
 * real[n_scenes][n_grid^3] and nearest: real[n_scenes][n_grid^3][3] written
 * (nearest = 0 where sdf stays inf); work: real[n_scenes][n_grid^3][4]
 * scratch.  Launches after the first iteration that changes no node return
 * at once (every later iteration would reproduce it). */
int mpm_target_sdf(MpmHandle* h, const void* target_density, void* target_sdf, void* nearest, void* work,
                   int32_t n_iters, void* stream);

/* compute_sdf_loss_kernel (loss.py:178-180) per scene, FP64 sum in a fixed
 * order: loss[s] = weight * sum_I target_sdf * grid_m (double[n_scenes],
 * overwritten).  If g_grid_m is not NULL, weight * target_sdf is ADDED to it,
 * so it can follow mpm_density_l1 (which overwrites). */
int mpm_sdf_loss(MpmHandle* h, const void* grid_m, const void* target_sdf, double weight, double* loss,
                 void* g_grid_m, void* stream);

/* iou_kernel (loss.py:294-308) per scene in FP64: ma = max(0, max m),
 * mb = max(0, max t), I = sum m t / ma / mb, U = sum m / ma + sum t / mb,
 * iou[s] = I / (U - I) (double[n_scenes]).  No adjoint: the reference's
 * iou_grad is empty (loss.py:318-321). */
int mpm_iou(MpmHandle* h, const void* grid_m, const void* target, double* iou, void* stream);

/* Hard contact distance (compute_contact_distance_kernel, loss.py:151-155,
 * started from 100000 as compute_loss_kernel does, loss.py:243-244):
 * min_dist[t] = min(100000, min_i max(sdf_t(x_i), 0)) over the particles of
 * tool t's scene (double[n_tools]); argmin[t] = the lowest particle index
 * attaining it, or -1 (int64[n_tools]).  Tools with action_dim 0 get 0 and -1
 * (Loss keeps movable tools only, loss.py:21-25). */
int mpm_contact_min_dist(MpmHandle* h, const void* state, const double* pose, double* min_dist, int64_t* argmin,
                         void* stream);
/* Adjoint: g_min_dist[t] flows to the particle argmin[t] (x rows of g_state,
 * accumulated) and to the tool pose (g_pose, double[n_tools][8],
 * accumulated) through max(sdf, 0), which passes it only where sdf > 0.
 * Ties send the whole gradient to the lowest index. */
int mpm_contact_min_dist_bwd(MpmHandle* h, const void* state, const double* pose, const int64_t* argmin,
                             const double* g_min_dist, void* g_state, double* g_pose, void* stream);

/* Per-particle tool distances (GradModel.compute_min_dist, function.py:79-89):
 * column c of out (real[n_cols][ld], n_cols from mpm_tool_distance_cols) holds
 * the SDF of the tool owning column c at every particle of that tool's scene
 * (Gripper: two columns, finger -1 then finger +1, as sdf_2 of
 * primitives.py:479-483), and 0 for particles of other scenes. */
int mpm_tool_distance_cols(MpmHandle* h);
int mpm_tool_distance(MpmHandle* h, const void* state, const double* pose, void* out, void* stream);
/* Adjoint (compute_min_dist.grad, function.py:154-159): accumulates the x
 * rows of g_state and g_pose (double[n_tools][8]) from g_out. */
int mpm_tool_distance_bwd(MpmHandle* h, const void* state, const double* pose, const void* g_out, void* g_state,
                          double* g_pose, void* stream);

/* Particle-SDF renderer (ParticleSDFRaster, taichi_three/tina/core/particle_sdf.py,
 * driven by plb/env_modeling/tina_renderer.py), as compute kernels writing
 * device buffers.  A volume (RENDERER.voxel_res / dx / bake_size of
 * plb/config/default_config.py:43-49; all buffers caller-owned device memory): */
typedef struct MpmRenderVolume {
  int32_t res[3];              /* voxels per axis (default 168^3) */
  int32_t bake_size;           /* splat radius in voxels (default 6) */
  double dx;                   /* voxel size (default 1/150) */
  unsigned long long* packed;  /* uint64[res] scratch: (quantised distance << 24) | rgb */
  float* sdf;                  /* float[res] baked SDF, smoothed twice */
  float* sdf_copy;             /* float[res] scratch */
  float* color;                /* float[res][3] */
  float* bbox;                 /* float[2][3]: lower and upper corner of the volume */
  int32_t* kbox;               /* int32[6] scratch */
} MpmRenderVolume;
/* One view (host struct): tina Engine's matrices and pixel sample offset. */
typedef struct MpmRenderView {
  float v2w[16], w2v[16];  /* Engine.V2W / W2V, row-major (camera = inverse(proj @ view)) */
  int32_t res[2];          /* image size (x, y); pixel (i, j) at i * res[1] + j */
  float bias[2];           /* sample offset in the pixel (0.5, 0.5 without TAA jitter) */
  float sdf_threshold;     /* RENDERER.sdf_threshold (default 0.37 * 0.56) */
  int32_t show_particles;  /* visualize_shape */
} MpmRenderView;

/* initialize_particles_kernel + build_sdf_from_particles (particle_sdf.py:548-568,
 * 237-265) for the particles of one scene: the volume's box from the
 * particles, a splat of (min(51 |voxel - p|, 255) << 24 | colour) by 64-bit
 * atomicMin over (-size-1 .. size]^3 voxels around each particle, the decode
 * into SDF / colour (bytes / 255) and two 27-point smoothings.  colors:
 * device uint32[n] of 0xRRGGBB for the scene's particles, NULL = white
 * (set_object).  A box larger than the volume (the reference asserts) sets
 * MPM_STATUS_RENDER_BOX; the particles outside are skipped. */
int mpm_render_bake(MpmHandle* h, const void* state, int32_t scene, const uint32_t* colors,
                    const MpmRenderVolume* vol, void* stream);
/* render_color + next_hit (particle_sdf.py:185-217, 353-440) for one scene:
 * per pixel the ground (view depth 0.99), the scene's tools sphere traced with
 * their SDFs at pose (double[n_tools][8], the frame rendered), and the baked
 * particle SDF marched with back-step refinement.  depth: float[res] view-space
 * z of the nearest hit; normal, color: float[res][3] (colour times 3, as
 * render_color scales it); tool_color: device float[n_tools][3]; image
 * (nullable): float[res][3] shaded as tina's Lighting.shade_color with
 * Diffuse (ambient 0.1 * colour + the light (1,2,3), colour 0.9, times colour / pi). */
int mpm_render_trace(MpmHandle* h, const MpmRenderVolume* vol, const MpmRenderView* view, int32_t scene,
                     const double* pose, const float* tool_color, float* depth, float* normal, float* color,
                     float* image, void* stream);

/* No counterpart in the reference.  One forward substep (as mpm_substep_fwd)
 * of a single scene that allocates nothing, for callers that cannot call
 * cudaMalloc: code stepping the scene from inside another framework's GPU
 * memory pool (which may hold nearly all of HBM and must not be bypassed),
 * or latency-bound loops that cannot afford the device-wide synchronisation
 * of cudaMalloc/cudaFree.  No handle: params (n_scenes = 1) and the host tool
 * table are passed per call; the caller still owns state_f, state_f1, pose_f
 * and pose_f1.  Grid scratch and tool table live in one file-scope static
 * device array of 20 MiB + 64 KiB, held by every GPU that loads the library
 * until the process exits.  Limits: n_particles <= 2^20; two grids of
 * n_grid^3 nodes within 16 MiB (n_grid <= 80 in FP32, <= 64 in FP64); at most
 * 8 tools, of types MPM_TOOL_SPHERE .. MPM_TOOL_GRIPPER (0-4) only.  Larger
 * sizes or other tool types return MPM_E_INVALID; the message is read with
 * mpm_last_error(NULL, ...).  The tool table is passed to the device by value
 * as a kernel parameter: a call issues kernel launches only, no host-to-device
 * copy.  status (may be NULL): a caller-owned 4-byte aligned device word into
 * which the call's kernels OR the MPM_STATUS_* bits (a particle stencil
 * outside the grid, skipped; a NaN/Inf); it is sticky, the caller clears and
 * reads it.  With NULL the bits go to a scratch word and are not reported.
 * The first call on a device performs set-up (cudaGetSymbolAddress on that
 * device and zeroing of the array's scene-index region); make that first call
 * before any stream capture.  All calls share the array: calls whose kernels
 * overlap on the GPU race, so serialise them. */
int mpm_substep_fwd_static(const MpmParams* params, const MpmToolDesc* tools, int32_t n_tools, const void* state_f,
                           void* state_f1, const double* pose_f, const double* pose_f1, uint32_t* status,
                           void* stream);

/* Reads the sticky device status word (synchronises the stream). */
int mpm_status(MpmHandle* h, uint32_t* status, int32_t clear, void* stream);
/* Copies the last error message of this handle (or of mpm_create if h is NULL). */
int mpm_last_error(MpmHandle* h, char* buf, size_t len);
/* Number of kernel launches issued through this handle since creation. */
int64_t mpm_launch_count(MpmHandle* h);

/* Kernel kinds reported by the profiler. */
#define MPM_K_P2G 0          /* p2g writing F' (forward)           */
#define MPM_K_P2G_RECOMP 1   /* p2g recomputing the grid (adjoint)  */
#define MPM_K_GRID_OP 2
#define MPM_K_G2P 3
#define MPM_K_G2P_ADJ 4
#define MPM_K_GRID_OP_ADJ 5
#define MPM_K_P2G_ADJ 6
#define MPM_K_CLEAR 7        /* grid clears (memset)               */
#define MPM_K_OTHER 8        /* density, loss, contact, tools       */
#define MPM_K_SORT 9         /* particle re-sort and its adjoint    */
#define MPM_K_COUNT 10

/* No counterpart in the reference (it has no profiler): when enabled, every
 * kernel launched through the handle is bracketed by a CUDA event pair on its
 * stream.  Not for use inside CUDA-graph capture. */
int mpm_profile_enable(MpmHandle* h, int32_t enable);
/* Synchronises, then writes per kind the summed device milliseconds and the
 * launch counts since the last read (arrays of MPM_K_COUNT), and resets. */
int mpm_profile_read(MpmHandle* h, double* ms, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* MPM_GB300_H */
