/*
 * braxg: C ABI of the GB300-native generalized-coordinates physics step.
 *
 * Drop-in boundary for brax's generalized pipeline:
 *   brax/generalized/pipeline.py:32-61   init(sys, q, qd)      -> braxg_init
 *   brax/generalized/pipeline.py:64-94   step(sys, state, act) -> braxg_step
 *   brax/envs/base.py:128-137            pipeline_step (n_frames x step with
 *                                        one action)            -> braxg_step
 *   lax.scan over env steps (brax/training/agents/apg/train.py:188-198)
 *                                                               -> braxg_rollout
 * The System pytree (brax/base.py:415-540) is passed once, packed by
 * brax_gb300/model_pack.py, to braxg_model_create.  The State pytree
 * (brax/generalized/base.py:25-92) is a struct of per-field device pointers,
 * env-major ([n_env, ...], float32, contiguous).
 *
 * All entry points are stream-ordered on the caller's cudaStream_t (passed as
 * void*), never synchronise the host, and allocate no device memory after
 * braxg_model_create.  Every call returns 0 on success or a braxg_status code;
 * braxg_last_error() returns a message for the calling thread's last failure.
 */
#ifndef BRAXG_H_
#define BRAXG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct braxg_model braxg_model;

enum braxg_status_code {
  BRAXG_OK = 0,
  BRAXG_ERR_INVALID = 1,     /* bad argument or descriptor (ValueError) */
  BRAXG_ERR_CUDA = 2,        /* a CUDA call failed (RuntimeError) */
  BRAXG_ERR_UNSUPPORTED = 3  /* model outside the supported envelope (NotImplementedError) */
};

/* How mass_mx_inv is produced after each step (brax/generalized/mass.py:86-106). */
enum braxg_inverse_mode {
  /* Newton-Schulz warm start from the previous inverse with the reference's
   * iteration count and best-iterate acceptance (brax/math.py:278-305). */
  BRAXG_INV_NEWTON_SCHULZ = 0,
  /* Exact SPD inverse (per-env symmetric Gauss-Jordan sweep; its pivots are
   * a Cholesky factorisation's, so a non-positive one flags the env). */
  BRAXG_INV_CHOLESKY = 1
};

/* Per-env status bits written to braxg_state.status. */
enum braxg_env_flags {
  BRAXG_ENV_NONFINITE = 1,   /* q or qd not finite after the call */
  BRAXG_ENV_NOT_SPD = 2,     /* a Cholesky pivot was <= 0 */
  BRAXG_ENV_NO_GRADIENT = 4, /* a step's projected-gradient tape was missing or inconsistent: no gradient */
  BRAXG_ENV_SKIPPED = 8,     /* not stepped: its batch work item did not fit the launch */
  BRAXG_ENV_BOUNDS = 16      /* checked build only: an arena, row or alignment check failed */
};

typedef struct {
  int32_t nl, nq, nv, nu, ncon, nlim, m;
} braxg_dims;

/* Fields of brax.generalized.base.State.  q, qd and mass_mx_inv are the
 * state carried between steps; every other pointer is an optional output
 * (NULL skips it). */
typedef struct {
  float* q;             /* [n, nq] */
  float* qd;            /* [n, nv] */
  float* mass_mx_inv;   /* [n, nv, nv] */
  float* x_pos;         /* [n, nl, 3] */
  float* x_rot;         /* [n, nl, 4] */
  float* xd_ang;        /* [n, nl, 3] */
  float* xd_vel;        /* [n, nl, 3] */
  float* qf_smooth;     /* [n, nv] */
  float* qf_constraint; /* [n, nv] */
  float* qdd;           /* [n, nv] */
  float* root_com;      /* [n, nl, 3] */
  float* cinr_pos;      /* [n, nl, 3]  cinr.transform.pos */
  float* cinr_rot;      /* [n, nl, 4]  cinr.transform.rot */
  float* cinr_i;        /* [n, nl, 9]  cinr.i */
  float* cd;            /* [n, nl, 6]  ang(3), vel(3) */
  float* cdof;          /* [n, nv, 6] */
  float* cdofd;         /* [n, nv, 6] */
  float* mass_mx;       /* [n, nv, nv] */
  float* con_jac;       /* [n, m, nv] */
  float* con_diag;      /* [n, m] */
  float* con_aref;      /* [n, m] */
  int32_t* status;      /* [n] braxg_env_flags */
  /* Optional [n, braxg_model_cache_words] cache (16-byte aligned) of every
   * position-level term of the state (the lagged terms the reference State
   * carries, brax/generalized/pipeline.py:79-92), written by the call that
   * produces the state.  A call whose input state carries it skips
   * recomputing those terms for every env whose q, qd (Newton-Schulz mode:
   * and mass_mx_inv) and per-env parameters equal the cached ones bit for bit
   * and whose cache was computed with the same threads_per_env (exact-inverse
   * mode: and an exact mass_mx_inv); other envs recompute them, so the result
   * is the same either way.  The cache belongs to the model that wrote it.
   * For models with more than 32 constraint rows whose arena that saves
   * shared memory, the output's cache also holds the step's Jacobian rows
   * beyond the first 32 while it runs (so more envs fit per CTA).  The
   * braxg_batch_* calls neither read nor write it. */
  float* cache;
  /* Optional contacts of the output state, contact.get(sys, state.x)
   * (brax/contact.py:28-67), which the reference adds to the State when
   * init / step run with debug=True (brax/generalized/pipeline.py:57-58,
   * 91-92): one entry per contact slot (mjx's fixed ncon), dist < 0 meaning
   * penetration, frame rows (normal, tangent1, tangent2) with the normal
   * pointing from geom1 to geom2.  The per-slot constants (geoms, friction,
   * solref, solimp, link_idx, elasticity) are the model's.  The braxg_batch_*
   * calls do not write them. */
  float* contact_dist;   /* [n, ncon] */
  float* contact_pos;    /* [n, ncon, 3] */
  float* contact_frame;  /* [n, ncon, 3, 3] */
  /* Optional solver diagnostic, no counterpart in the reference (jaxopt
   * returns no state there): per env, the number of the call's pipeline
   * steps whose projected-gradient solve (brax/generalized/constraint.py:
   * 229-238) stopped at solver_iterations with its error still above tol. */
  int32_t* solver_maxiter;  /* [n] */
} braxg_state;

/* Per-stage profile slots of braxg_options.stage_cycles (sums over envs of
 * clock64 deltas taken by lane 0 of each env's team, plus event counters). */
enum braxg_profile_slot {
  BRAXG_PROF_FK = 0, BRAXG_PROF_COM, BRAXG_PROF_CRBA, BRAXG_PROF_INVERSE,
  BRAXG_PROF_JACOBIAN, BRAXG_PROF_SMOOTH, BRAXG_PROF_CONSTRAINT, BRAXG_PROF_INTEGRATE,
  BRAXG_PROF_IO, BRAXG_PROF_MATVECS, BRAXG_PROF_ROWS, BRAXG_PROF_NS_RESETS,
  BRAXG_PROF_SUBSTEPS,
  /* braxg_rollout_vjp phases: checkpoint pass, segment recompute, per-frame
   * restore, and the reverse stages */
  BRAXG_PROF_VJP_CHECKPOINT = 16, BRAXG_PROF_VJP_RECOMPUTE, BRAXG_PROF_VJP_RESTORE,
  BRAXG_PROF_REV_INTEGRATE, BRAXG_PROF_REV_QDD, BRAXG_PROF_REV_CONSTRAINT, BRAXG_PROF_REV_SMOOTH,
  BRAXG_PROF_REV_INVERSE, BRAXG_PROF_REV_CRBA, BRAXG_PROF_REV_ROWS, BRAXG_PROF_REV_COM,
  BRAXG_PROF_REV_FK,
  /* explicit projected-gradient solve: forming W, A, b / iterating */
  BRAXG_PROF_PG_BUILD = 28, BRAXG_PROF_PG_ITERATE,
  BRAXG_PROF_SLOTS = 32
};

/* Per-env System parameters (the fields brax's DomainRandomizationVmapWrapper,
 * brax/envs/wrappers/training.py:223-260, vmaps over; System leaves of
 * brax/base.py:415-540): each pointer is [n, k] device memory overriding the
 * model's value for every env, or NULL to keep the model's.  Forward paths
 * of single-model calls only (init, step, rollout, env rollout); gradients
 * and batches use the model's values.  The dynamics fields (link masses and
 * inertias, dof armature, damping and stiffness) take an extra per-env
 * region of the kernel's shared-memory arena, only in calls that pass one of
 * them.  Fluid forces keep the model's inertia-equivalent boxes. */
typedef struct {
  const float* friction;       /* [n, ncon] sliding friction of every contact slot */
  const float* act_gain;       /* [n, nu] actuator gain */
  const float* act_bias_q;     /* [n, nu] actuator bias on q */
  const float* act_bias_qd;    /* [n, nu] actuator bias on qd */
  const float* link_mass;      /* [n, nl] link.inertia.mass */
  const float* link_inertia;   /* [n, nl, 3, 3] link.inertia.i */
  const float* dof_armature;   /* [n, nv] dof.armature */
  const float* dof_damping;    /* [n, nv] dof.damping */
  const float* dof_stiffness;  /* [n, nv] dof.stiffness */
} braxg_randomization;

typedef struct {
  int32_t inverse_mode;     /* braxg_inverse_mode */
  int32_t threads_per_env;  /* 0 = tuned, else 16 or 32 lanes per env */
  int32_t envs_per_cta;     /* 0 = tuned */
  /* CTA barriers skipped between stages (bit 0: after the constraint solve,
   * bit 1: after the integrator).  Teams never share data, so this changes
   * no result, only how far the envs of a CTA may drift apart: 0 keeps
   * every stage in lockstep. */
  int32_t relax_barriers;
  /* Optional device buffer of BRAXG_PROF_SLOTS uint64 counters the kernel
   * adds its per-stage cycle counts into (NULL = no profiling). */
  unsigned long long* stage_cycles;
  /* Optional per-env System parameters (NULL = the model's for every env). */
  const braxg_randomization* randomization;
} braxg_options;

/* Copies a packed System descriptor to `device`.  Replaces tracing the
 * System pytree into the jitted step (brax/io/mjcf.py:317-489 builds it). */
int braxg_model_create(const void* desc, size_t desc_bytes, int device, braxg_model** out);
int braxg_model_destroy(braxg_model* model);
int braxg_model_dims(const braxg_model* model, braxg_dims* out);
/* Floats per env of braxg_state.cache for this model. */
int braxg_model_cache_words(const braxg_model* model, int32_t* words);

/* Floats per env that a call actually reads from and writes to the caches:
 * `fixed_words`, plus `row_words` for every active constraint row beyond the
 * first `rows_in_fixed`. */
int braxg_model_cache_span(const braxg_model* model, int32_t* fixed_words, int32_t* row_words,
                           int32_t* rows_in_fixed);

/* brax/generalized/pipeline.py:32-61.  Reads q [n, nq], qd [n, nv]; writes the
 * State fields of `out` (mass_mx_inv is the exact SPD inverse, the forces are
 * zero). */
int braxg_init(const braxg_model* model, void* stream, int n_env, const float* q,
               const float* qd, braxg_state* out, const braxg_options* opt);

/* n_frames x brax/generalized/pipeline.py:64-94 with one action per env
 * (brax/envs/base.py:128-137).  act is [n, nu] (NULL = no actuation).  Reads
 * in->q, in->qd, in->mass_mx_inv; `out` may alias `in`. */
int braxg_step(const braxg_model* model, void* stream, int n_env, int n_frames,
               const float* act, const braxg_state* in, braxg_state* out,
               const braxg_options* opt);

/* n_steps env steps of n_frames pipeline steps each, act_seq [n_steps, n, nu].
 * traj_q [n_steps, n, nq] and traj_qd [n_steps, n, nv] (optional) receive the
 * state after every env step; `out` receives the final state. */
int braxg_rollout(const braxg_model* model, void* stream, int n_env, int n_steps,
                  int n_frames, const float* act_seq, const braxg_state* in,
                  braxg_state* out, float* traj_q, float* traj_qd,
                  const braxg_options* opt);

/* ---- Fused env step ---------------------------------------------------------
 * The locomotion task of brax/envs/ant.py:233-279 (forward reward, healthy
 * reward, control cost, healthy-z termination, obs = q[2:] ++ qd) wrapped by
 * EpisodeWrapper and AutoResetWrapper (brax/envs/wrappers/training.py:75-158),
 * computed in the same launch as the physics: per env step, the n_frames
 * pipeline steps, then reward / done / metrics, then (done envs) the reset to
 * the episode's first state. */
typedef struct {
  float ctrl_cost_weight;            /* 0.5 */
  float healthy_reward;              /* 1.0 */
  float healthy_z_min, healthy_z_max;  /* 0.2, 1.0: torso (link 0) height range */
  int32_t terminate_when_unhealthy;  /* 1 */
  int32_t exclude_current_positions; /* 1: obs = q[2:] ++ qd, else q ++ qd */
  int32_t episode_length;            /* 1000 env steps (EpisodeWrapper) */
  int32_t action_repeat;             /* 1 */
  int32_t auto_reset;                /* 1 (AutoResetWrapper) */
  int32_t reserved[3];
} braxg_task;

/* Metric columns of braxg_env_io.metrics (ant.py:256-267 order). */
enum braxg_env_metric {
  BRAXG_M_REWARD_FORWARD = 0, BRAXG_M_REWARD_SURVIVE, BRAXG_M_REWARD_CTRL,
  BRAXG_M_REWARD_CONTACT, BRAXG_M_X_POSITION, BRAXG_M_Y_POSITION,
  BRAXG_M_DISTANCE_FROM_ORIGIN, BRAXG_M_X_VELOCITY, BRAXG_M_Y_VELOCITY,
  BRAXG_M_FORWARD_REWARD, BRAXG_M_COUNT = 10
};

/* Per-env task buffers (device pointers).  steps, truncation and done carry the
 * wrappers' state between calls (read and written); first_* is the state an
 * auto-reset returns to (the episode's first pipeline state). */
typedef struct {
  float* obs;          /* [n, obs_size] after the last env step (post-reset) */
  float* reward;       /* [n_steps, n] */
  float* done;         /* [n_steps, n] (optional) */
  float* metrics;      /* [n, BRAXG_M_COUNT] of the last env step (optional) */
  float* steps;        /* [n] episode step counter */
  float* truncation;   /* [n] */
  float* last_done;    /* [n] done of the previous env step (in) / last (out) */
  const float* first_q;            /* [n, nq] */
  const float* first_qd;           /* [n, nv] */
  const float* first_mass_mx_inv;  /* [n, nv, nv] (Newton-Schulz mode) */
} braxg_env_io;

/* n_steps env steps (env.step of AutoResetWrapper(EpisodeWrapper(task))) with
 * act_seq [n_steps, n, nu]; the pipeline state in/out as braxg_rollout. */
int braxg_env_rollout(const braxg_model* model, void* stream, int n_env, int n_steps,
                      int n_frames, const float* act_seq, const braxg_state* in,
                      braxg_state* out, const braxg_task* task, const braxg_env_io* io,
                      const braxg_options* opt);

/* Smallest device workspace braxg_rollout_vjp accepts: the checkpoints (every
 * ckpt_every env steps) and the frame states and frame snapshots of one
 * segment; every segment but the last is then recomputed. */
int braxg_rollout_vjp_workspace(const braxg_model* model, int n_env, int n_steps, int n_frames,
                                int ckpt_every, size_t* bytes);

/* Workspace that keeps the last `resident` segments' frame snapshots from the
 * checkpoint pass (resident <= 0: all segments, no recompute at all).
 * braxg_rollout_vjp keeps as many trailing segments resident as the
 * workspace it is given holds, so more memory means less recompute; the
 * gradient is the same either way. */
int braxg_rollout_vjp_workspace_resident(const braxg_model* model, int n_env, int n_steps,
                                         int n_frames, int ckpt_every, int resident,
                                         size_t* bytes);

/* The same for an inverse mode: BRAXG_INV_NEWTON_SCHULZ (on a model with
 * Newton-Schulz iterations) needs more (the carried inverse in every
 * checkpoint, each snapshotted frame's update record, the reverse's scratch);
 * the other sizes above are for the exact inverse. */
int braxg_rollout_vjp_workspace_mode(const braxg_model* model, int n_env, int n_steps,
                                     int n_frames, int ckpt_every, int resident, int inverse_mode,
                                     size_t* bytes);

/* Gradient of a rollout (the reverse of braxg_rollout), the replacement for
 * jax.grad through lax.scan of pipeline_step (brax/training/agents/apg/
 * train.py:188-198).  Runs the forward from (q0, qd0) with act_seq
 * [n_steps, n, nu], checkpointing every ckpt_every env steps, then the
 * hand-written reverse of every pipeline step, recomputing the segments whose
 * frame snapshots the workspace cannot hold.  q_bar / qd_bar
 * [n_steps, n, nq|nv] are the loss cotangents of the state after each env step
 * (NULL = zero); outputs are act_bar [n_steps, n, nu], q0_bar [n, nq],
 * qd0_bar [n, nv] and, optionally, the forward trajectory traj_q / traj_qd.
 * The mass-matrix inverse is exact (Cholesky) unless opt->inverse_mode is
 * BRAXG_INV_NEWTON_SCHULZ on a model with Newton-Schulz iterations: then the
 * rollout carries the reference's inverse (exact at the first frame, as
 * pipeline.init computes it; updated by Newton-Schulz every frame after,
 * brax/generalized/mass.py:99-101) and the reverse differentiates through
 * those updates (brax/math.py:278-305, as jax.grad does; workspace from
 * braxg_rollout_vjp_workspace_mode; the reverse of each update also takes
 * shared memory per env: 12 KB up to 16 dofs, 48 KB up to 32, so a model
 * that no longer fits the launch gets BRAXG_ERR_UNSUPPORTED in that mode
 * only).  Status bits as braxg_env_flags.
 * Supports hinge/slide/free joints, every contact kind of the forward
 * (world-plane sphere, capsule and box; sphere / capsule pairs between two
 * moving geoms), joint limits and fluid drag, with either constraint-solve
 * path (A formed explicitly up to 32 active rows, applied implicitly above). */
int braxg_rollout_vjp(const braxg_model* model, void* stream, int n_env, int n_steps, int n_frames,
                      int ckpt_every, const float* act_seq, const float* q0, const float* qd0,
                      const float* q_bar, const float* qd_bar, float* act_bar, float* q0_bar,
                      float* qd0_bar, float* traj_q, float* traj_qd, void* workspace,
                      size_t workspace_bytes, int32_t* status, const braxg_options* opt);

/* braxg_rollout_vjp split in two launches, for a custom_vjp whose forward
 * output is needed before the cotangents exist (jax.custom_vjp fwd / bwd of
 * the scan, a torch.autograd.Function's forward / backward, the closed loop
 * of brax/training/agents/apg/train.py:179-236 where each env step's
 * cotangent comes back through the policy).  braxg_rollout_vjp_fwd runs the
 * forward: traj_q / traj_qd [n_steps, n, nq|nv] (required) and the
 * checkpoints and frame snapshots in the workspace (sized as for
 * braxg_rollout_vjp; segments the workspace cannot keep resident are
 * recomputed by the reverse); status gets the forward's bits.
 * braxg_rollout_vjp_bwd then runs only the reverse and must get the same
 * model, sizes, act_seq, q0, qd0 and the workspace (pointer and size) of the
 * forward call, untouched since; it ORs its bits into status.  Together they
 * give bitwise the gradient and trajectory of one braxg_rollout_vjp call, and
 * the reverse does not recompute the resident segments' forward. */
int braxg_rollout_vjp_fwd(const braxg_model* model, void* stream, int n_env, int n_steps, int n_frames,
                          int ckpt_every, const float* act_seq, const float* q0, const float* qd0,
                          float* traj_q, float* traj_qd, void* workspace, size_t workspace_bytes,
                          int32_t* status, const braxg_options* opt);
int braxg_rollout_vjp_bwd(const braxg_model* model, void* stream, int n_env, int n_steps, int n_frames,
                          int ckpt_every, const float* act_seq, const float* q0, const float* qd0,
                          const float* q_bar, const float* qd_bar, float* act_bar, float* q0_bar,
                          float* qd0_bar, void* workspace, size_t workspace_bytes, int32_t* status,
                          const braxg_options* opt);

/* braxg_rollout_vjp without a workspace argument, for callers that cannot
 * allocate device memory: an XLA custom call registered without access to the
 * scratch allocator, a plugin whose host framework owns every device
 * allocation, or a control loop that must not enter the CUDA allocator.  The
 * checkpoint / segment scratch is one fixed 8 MiB array inside this library
 * (braxg_rollout_vjp_noalloc_capacity() bytes), held by every device that
 * loads the library until the process exits; requests needing more
 * (braxg_rollout_vjp_workspace) fail with BRAXG_ERR_INVALID.  Nothing is
 * allocated or freed.  The first call on a device looks up the array's device
 * address with that device current, so make one call on each device before
 * any stream capture; the address is kept for the process, so after
 * cudaDeviceReset (which also invalidates every model handle) the entry point
 * must not be called again.  All calls share the one array: calls that overlap on
 * the GPU (different streams, or different threads without ordering) race on
 * it and corrupt each other's gradients.  No counterpart in the reference: it
 * exists only for callers that cannot allocate. */
size_t braxg_rollout_vjp_noalloc_capacity(void);
int braxg_rollout_vjp_noalloc(const braxg_model* model, void* stream, int n_env, int n_steps,
                              int n_frames, int ckpt_every, const float* act_seq, const float* q0,
                              const float* qd0, const float* q_bar, const float* qd_bar,
                              float* act_bar, float* q0_bar, float* qd0_bar, float* traj_q,
                              float* traj_qd, int32_t* status, const braxg_options* opt);

/* ---- Uneven batches --------------------------------------------------------
 * Envs of several models (different nv, link counts and contact sets) stepped
 * by ONE persistent launch.  The reference steps one System per jitted
 * function (jax.vmap over envs of the same System, brax/envs/wrappers/
 * training.py:66-72); a batch of different Systems has no counterpart there
 * and would be one jitted step per System.  Each model keeps the meaning of
 * braxg_step/braxg_rollout for its own envs.
 *
 * State arrays are flat: model g's envs occupy one contiguous run of every
 * field, starting at braxg_batch_get_offsets(batch, g) in units of that field's
 * per-env size class; the offsets of index n_models are the totals.
 *
 * Calls on ONE batch must be stream-ordered (one stream, or streams ordered
 * by events; a replay of a captured graph counts as a call): every launch
 * zeroes and then draws work items from the batch's one device counter, so
 * two launches of the same batch running at the same time skip or repeat
 * each other's items and give wrong results with no error.  Different
 * batches are independent. */
typedef struct braxg_batch braxg_batch;

/* Launch shape for the models with nv <= nv_max (the first matching entry
 * applies; models matching none get the single-model default: 16 lanes for
 * nv <= 8, else 32, and envs_per_cta 0). */
typedef struct {
  int32_t nv_max;
  int32_t threads_per_env;  /* 16 or 32 */
  int32_t envs_per_cta;     /* envs of one model per CTA work item; 0 = as many as fit */
  int32_t reserved;
} braxg_bucket_shape;

typedef struct {
  int64_t env;      /* status; env index */
  int64_t q;        /* q, traj_q (x1) */
  int64_t qd;       /* qd, qf_smooth, qf_constraint, qdd, traj_qd (x1); cdof, cdofd (x6) */
  int64_t mass_mx;  /* mass_mx, mass_mx_inv (x1) */
  int64_t link;     /* x_pos, xd_ang, xd_vel, root_com, cinr_pos (x3); x_rot, cinr_rot (x4);
                       cd (x6); cinr_i (x9) */
  int64_t act;      /* act (x1) */
  int64_t row;      /* con_diag, con_aref (x1) */
  int64_t jac;      /* con_jac (x1) */
} braxg_batch_offsets;

/* Builds the work list of a batch: n_env[g] envs of models[g] (all on one
 * device), n_frames[g] pipeline steps per env step (NULL = 1 each).  Work items
 * are CTA-sized groups of envs of one model, ordered by decreasing estimated
 * cost and taken from a device counter by a grid of (SMs x resident CTAs)
 * persistent CTAs.  smem_per_cta = 0 allows the whole 227 KB (one CTA per
 * SM, all its warps on the same stage's code); a non-zero value is a limit,
 * and a shape that does not fit it is BRAXG_ERR_INVALID.  Allocates the device work list; later calls allocate
 * nothing. */
int braxg_batch_create(const braxg_model* const* models, const int32_t* n_env,
                       const int32_t* n_frames, int n_models,
                       const braxg_bucket_shape* shapes, int n_shapes,
                       int32_t smem_per_cta, braxg_batch** out);
int braxg_batch_destroy(braxg_batch* batch);
int braxg_batch_get_offsets(const braxg_batch* batch, int index, braxg_batch_offsets* out);
int braxg_batch_launch_info(const braxg_batch* batch, int32_t* grid, int32_t* block,
                            int32_t* smem_bytes, int32_t* n_items);

/* braxg_init for every env of the batch (flat q, qd and out fields). */
int braxg_batch_init(const braxg_batch* batch, void* stream, const float* q,
                     const float* qd, braxg_state* out, const braxg_options* opt);

/* braxg_rollout for every env of the batch: act_seq [n_steps, total act],
 * traj_q [n_steps, total q], traj_qd [n_steps, total qd] (optional).  One
 * kernel launch plus one 4-byte memset of the work counter on `stream`; both
 * are stream-ordered, so the call can be captured into a CUDA graph. */
int braxg_batch_rollout(const braxg_batch* batch, void* stream, int n_steps,
                        const float* act_seq, const braxg_state* in, braxg_state* out,
                        float* traj_q, float* traj_qd, const braxg_options* opt);

/* Launch shape a braxg_init / braxg_step / braxg_rollout / braxg_env_rollout
 * call of n_env envs takes for this model (n_env 0: the largest CTA) when its
 * output state carries a cache (see braxg_state.cache): lanes per env, envs
 * per CTA, dynamic shared memory bytes per CTA. */
int braxg_launch_shape(const braxg_model* model, const braxg_options* opt, int n_env,
                       int32_t* threads_per_env, int32_t* envs_per_cta,
                       int32_t* smem_bytes);

/* Number of kernel launches the last successful call on this thread issued. */
int braxg_last_launch_count(void);

const char* braxg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* BRAXG_H_ */
