// The work behind the XLA FFI handlers of braxg_xla.cc: shape checks of the
// buffers XLA passes and the braxg C ABI calls they turn into.  Plain C++
// (no XLA types), so that the same code also compiles against a stub of the
// braxg calls for a host-only test.
//
// Batching follows jax.vmap over the reference's per-env functions
// (brax/envs/wrappers/training.py:66-72): a per-env array of trailing shape
// S arrives as [..., S]; its leading dimensions are the env batch (none: one
// env, an unbatched call), and every argument of one call must agree on it.
#pragma once
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <string>

#include "braxg.h"

namespace braxg_xla {

// An XLA buffer as the handlers see it.
struct Buf {
  void* data;
  const int64_t* dims;
  int rank;
  float* f() const { return static_cast<float*>(data); }
};

// Envs of `b` if its trailing dimensions (after `skip` leading ones, e.g. the
// time axis of a sequence) are `tail`: the product of the dimensions between;
// -1 if they do not match.
inline int64_t envs_of(const Buf& b, std::initializer_list<int64_t> tail, int skip = 0) {
  const int nt = static_cast<int>(tail.size());
  if (b.rank < skip + nt) return -1;
  int k = b.rank - nt;
  for (int64_t t : tail)
    if (b.dims[k++] != t) return -1;
  int64_t n = 1;
  for (int i = skip; i < b.rank - nt; ++i) n *= b.dims[i];
  return n;
}

inline std::string dims_str(const Buf& b) {
  std::string s = "[";
  for (int i = 0; i < b.rank; ++i) s += (i ? ", " : "") + std::to_string(b.dims[i]);
  return s + "]";
}

// Checks that `b` is a batch of `n` envs (n < 0: takes its count) of trailing
// shape `tail`; returns "" or the error.
inline std::string expect(const char* name, const Buf& b, std::initializer_list<int64_t> tail, int64_t& n,
                          int skip = 0) {
  const int64_t e = envs_of(b, tail, skip);
  std::string want;
  for (int64_t t : tail) want += ", " + std::to_string(t);
  if (e < 0) return std::string(name) + " has shape " + dims_str(b) + ", expected [..." + want + "]";
  if (n >= 0 && e != n)
    return std::string(name) + " holds " + std::to_string(e) + " envs, expected " + std::to_string(n);
  n = e;
  return "";
}

inline std::string last_error(const char* call, int rc) {
  const char* m = braxg_last_error();
  return std::string(call) + " failed (" + std::to_string(rc) + "): " + (m ? m : "");
}

#define BRAXG_XLA_TRY(expr)           \
  do {                                \
    std::string e_ = (expr);          \
    if (!e_.empty()) return e_;       \
  } while (0)

// pipeline.step (brax/generalized/pipeline.py:64-94) x n_frames with one
// action (brax/envs/base.py:128-137).  In: q [.., nq], qd [.., nv],
// mass_mx_inv [.., nv, nv], act [.., nu].  Out: q, qd, mass_mx_inv, x_pos
// [.., nl, 3], x_rot [.., nl, 4], xd_ang, xd_vel [.., nl, 3], qf_smooth,
// qf_constraint, qdd [.., nv], status (int32) [..].
inline std::string step(const braxg_model* m, void* stream, int n_frames, int inverse_mode, const Buf& q,
                        const Buf& qd, const Buf& minv, const Buf& act, const Buf& q_out, const Buf& qd_out,
                        const Buf& minv_out, const Buf& x_pos, const Buf& x_rot, const Buf& xd_ang,
                        const Buf& xd_vel, const Buf& qf_smooth, const Buf& qf_constraint, const Buf& qdd,
                        const Buf& status) {
  braxg_dims d;
  int rc = braxg_model_dims(m, &d);
  if (rc) return last_error("braxg_model_dims", rc);
  int64_t n = -1;
  BRAXG_XLA_TRY(expect("q", q, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd", qd, {d.nv}, n));
  BRAXG_XLA_TRY(expect("mass_mx_inv", minv, {d.nv, d.nv}, n));
  BRAXG_XLA_TRY(expect("act", act, {d.nu}, n));
  BRAXG_XLA_TRY(expect("q_out", q_out, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd_out", qd_out, {d.nv}, n));
  BRAXG_XLA_TRY(expect("mass_mx_inv_out", minv_out, {d.nv, d.nv}, n));
  BRAXG_XLA_TRY(expect("x_pos", x_pos, {d.nl, 3}, n));
  BRAXG_XLA_TRY(expect("x_rot", x_rot, {d.nl, 4}, n));
  BRAXG_XLA_TRY(expect("xd_ang", xd_ang, {d.nl, 3}, n));
  BRAXG_XLA_TRY(expect("xd_vel", xd_vel, {d.nl, 3}, n));
  BRAXG_XLA_TRY(expect("qf_smooth", qf_smooth, {d.nv}, n));
  BRAXG_XLA_TRY(expect("qf_constraint", qf_constraint, {d.nv}, n));
  BRAXG_XLA_TRY(expect("qdd", qdd, {d.nv}, n));
  BRAXG_XLA_TRY(expect("status", status, {}, n));
  if (n > INT32_MAX) return "too many envs in one call";
  braxg_state in{}, out{};
  in.q = q.f();
  in.qd = qd.f();
  in.mass_mx_inv = minv.f();
  out.q = q_out.f();
  out.qd = qd_out.f();
  out.mass_mx_inv = minv_out.f();
  out.x_pos = x_pos.f();
  out.x_rot = x_rot.f();
  out.xd_ang = xd_ang.f();
  out.xd_vel = xd_vel.f();
  out.qf_smooth = qf_smooth.f();
  out.qf_constraint = qf_constraint.f();
  out.qdd = qdd.f();
  out.status = static_cast<int32_t*>(status.data);
  braxg_options opt{};
  opt.inverse_mode = inverse_mode;
  rc = braxg_step(m, stream, static_cast<int>(n), n_frames, d.nu ? act.f() : nullptr, &in, &out, &opt);
  return rc ? last_error("braxg_step", rc) : "";
}

// lax.scan of env steps: act_seq [T, .., nu] from (q0, qd0) (the state of
// pipeline.init), trajectory traj_q [T, .., nq], traj_qd [T, .., nv] after every
// env step, status [..].
inline std::string rollout(const braxg_model* m, void* stream, int n_frames, int inverse_mode, const Buf& q0,
                           const Buf& qd0, const Buf& act_seq, const Buf& traj_q, const Buf& traj_qd,
                           const Buf& status, float* scratch_state, size_t scratch_floats) {
  braxg_dims d;
  int rc = braxg_model_dims(m, &d);
  if (rc) return last_error("braxg_model_dims", rc);
  int64_t n = -1;
  BRAXG_XLA_TRY(expect("q0", q0, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd0", qd0, {d.nv}, n));
  BRAXG_XLA_TRY(expect("act_seq", act_seq, {d.nu}, n, 1));
  BRAXG_XLA_TRY(expect("traj_q", traj_q, {d.nq}, n, 1));
  BRAXG_XLA_TRY(expect("traj_qd", traj_qd, {d.nv}, n, 1));
  BRAXG_XLA_TRY(expect("status", status, {}, n));
  if (act_seq.rank < 1 || traj_q.rank < 1 || traj_qd.rank < 1 || traj_q.dims[0] != act_seq.dims[0] ||
      traj_qd.dims[0] != act_seq.dims[0])
    return "act_seq, traj_q and traj_qd must share their leading (time) dimension";
  const int64_t T = act_seq.dims[0];
  if (n > INT32_MAX || T > INT32_MAX) return "too many envs or steps in one call";
  // the initial state's mass_mx_inv (exact, from braxg_init) and the final
  // state live in caller scratch: [n, nv, nv] each for the init and out states
  const size_t need = 2 * static_cast<size_t>(n) * d.nv * d.nv;
  if (scratch_state == nullptr || scratch_floats < need) return "rollout scratch too small";
  braxg_state s0{}, s1{};  // only mass_mx_inv and status are written
  s0.mass_mx_inv = scratch_state;
  s0.status = static_cast<int32_t*>(status.data);
  braxg_options opt{};
  opt.inverse_mode = inverse_mode;
  if (n > 0) {
    rc = braxg_init(m, stream, static_cast<int>(n), q0.f(), qd0.f(), &s0, &opt);
    if (rc) return last_error("braxg_init", rc);
  }
  if (T == 0 || n == 0) return "";
  // the rollout reads the initial state from q0 / qd0 and init's inverse
  braxg_state in{};
  in.q = q0.f();
  in.qd = qd0.f();
  in.mass_mx_inv = scratch_state;
  s1.mass_mx_inv = scratch_state + static_cast<size_t>(n) * d.nv * d.nv;
  s1.status = static_cast<int32_t*>(status.data);
  rc = braxg_rollout(m, stream, static_cast<int>(n), static_cast<int>(T), n_frames, d.nu ? act_seq.f() : nullptr,
                     &in, &s1, traj_q.f(), traj_qd.f(), &opt);
  return rc ? last_error("braxg_rollout", rc) : "";
}

// Scratch floats `rollout` needs for n envs.
inline size_t rollout_scratch_floats(const braxg_model* m, int64_t n) {
  braxg_dims d;
  if (braxg_model_dims(m, &d)) return 0;
  return 2 * static_cast<size_t>(n) * d.nv * d.nv;
}

// Workspace bytes of rollout_vjp for these buffers (0 on a shape error);
// inverse_mode as braxg_options.inverse_mode.
inline size_t rollout_vjp_workspace(const braxg_model* m, int n_frames, int ckpt_every, const Buf& q0,
                                    const Buf& act_seq, int inverse_mode = BRAXG_INV_CHOLESKY) {
  braxg_dims d;
  if (braxg_model_dims(m, &d)) return 0;
  const int64_t n = envs_of(q0, {d.nq});
  if (n < 0 || act_seq.rank < 1) return 0;
  size_t bytes = 0;
  if (braxg_rollout_vjp_workspace_mode(m, static_cast<int>(n), static_cast<int>(act_seq.dims[0]), n_frames,
                                       ckpt_every, 1, inverse_mode, &bytes))
    return 0;
  return bytes;
}

// The reverse of `rollout` (jax.grad through lax.scan of pipeline_step,
// brax/training/agents/apg/train.py:188-198): cotangents q_bar [T, .., nq],
// qd_bar [T, .., nv] of the trajectory give act_bar [T, .., nu], q0_bar, qd0_bar.
// With workspace == nullptr it uses the library's fixed scratch
// (braxg_rollout_vjp_noalloc) for handlers that got no scratch allocator.
inline std::string rollout_vjp(const braxg_model* m, void* stream, int n_frames, int ckpt_every, const Buf& q0,
                               const Buf& qd0, const Buf& act_seq, const Buf& q_bar, const Buf& qd_bar,
                               const Buf& act_bar, const Buf& q0_bar, const Buf& qd0_bar, const Buf& status,
                               void* workspace, size_t workspace_bytes, int inverse_mode = BRAXG_INV_CHOLESKY) {
  braxg_dims d;
  int rc = braxg_model_dims(m, &d);
  if (rc) return last_error("braxg_model_dims", rc);
  int64_t n = -1;
  BRAXG_XLA_TRY(expect("q0", q0, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd0", qd0, {d.nv}, n));
  BRAXG_XLA_TRY(expect("act_seq", act_seq, {d.nu}, n, 1));
  BRAXG_XLA_TRY(expect("q_bar", q_bar, {d.nq}, n, 1));
  BRAXG_XLA_TRY(expect("qd_bar", qd_bar, {d.nv}, n, 1));
  BRAXG_XLA_TRY(expect("act_bar", act_bar, {d.nu}, n, 1));
  BRAXG_XLA_TRY(expect("q0_bar", q0_bar, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd0_bar", qd0_bar, {d.nv}, n));
  BRAXG_XLA_TRY(expect("status", status, {}, n));
  const int64_t T = act_seq.dims[0];
  if (q_bar.dims[0] != T || qd_bar.dims[0] != T || act_bar.dims[0] != T)
    return "act_seq, q_bar, qd_bar and act_bar must share their leading (time) dimension";
  if (n > INT32_MAX || T > INT32_MAX || T < 1) return "the rollout needs 1 .. 2^31-1 steps and envs";
  braxg_options opt{};
  opt.inverse_mode = inverse_mode;
  float* ab = d.nu ? act_bar.f() : nullptr;
  const float* as = d.nu ? act_seq.f() : nullptr;
  if (workspace == nullptr) {
    rc = braxg_rollout_vjp_noalloc(m, stream, static_cast<int>(n), static_cast<int>(T), n_frames, ckpt_every, as,
                                   q0.f(), qd0.f(), q_bar.f(), qd_bar.f(), ab, q0_bar.f(), qd0_bar.f(), nullptr,
                                   nullptr, static_cast<int32_t*>(status.data), &opt);
    return rc ? last_error("braxg_rollout_vjp_noalloc", rc) : "";
  }
  rc = braxg_rollout_vjp(m, stream, static_cast<int>(n), static_cast<int>(T), n_frames, ckpt_every, as, q0.f(),
                         qd0.f(), q_bar.f(), qd_bar.f(), ab, q0_bar.f(), qd0_bar.f(), nullptr, nullptr, workspace,
                         workspace_bytes, static_cast<int32_t*>(status.data), &opt);
  return rc ? last_error("braxg_rollout_vjp", rc) : "";
}

// Bytes of the residual rollout_vjp_fwd leaves for rollout_vjp_bwd: the
// gradient workspace with every checkpoint segment resident, so that the
// reverse only reads it (0 on a shape error).
inline size_t rollout_vjp_residual_bytes(const braxg_model* m, int n_frames, int ckpt_every, const Buf& q0,
                                         const Buf& act_seq, int inverse_mode = BRAXG_INV_CHOLESKY) {
  braxg_dims d;
  if (braxg_model_dims(m, &d)) return 0;
  const int64_t n = envs_of(q0, {d.nq});
  if (n < 0 || act_seq.rank < 1) return 0;
  size_t bytes = 0;
  if (braxg_rollout_vjp_workspace_mode(m, static_cast<int>(n), static_cast<int>(act_seq.dims[0]), n_frames,
                                       ckpt_every, 0, inverse_mode, &bytes))
    return 0;
  return bytes;
}

// Checks the residual buffer (uint8 [bytes]) against what the sizes need.
inline std::string expect_residual(const braxg_model* m, int n_frames, int ckpt_every, const Buf& q0,
                                   const Buf& act_seq, const Buf& residual, int inverse_mode) {
  const size_t need = rollout_vjp_residual_bytes(m, n_frames, ckpt_every, q0, act_seq, inverse_mode);
  if (need == 0) return "cannot size the gradient residual for q0 " + dims_str(q0);
  if (residual.rank != 1 || static_cast<size_t>(residual.dims[0]) < need)
    return "residual has shape " + dims_str(residual) + ", expected [" + std::to_string(need) + "]";
  return "";
}

// jax.custom_vjp forward of the rollout: the trajectory traj_q [T, .., nq],
// traj_qd [T, .., nv], status [..], and the residual (the forward's
// checkpoints and frame snapshots) for rollout_vjp_bwd; inverse_mode as
// braxg_options.inverse_mode (the same for both halves).
inline std::string rollout_vjp_fwd(const braxg_model* m, void* stream, int n_frames, int ckpt_every, const Buf& q0,
                                   const Buf& qd0, const Buf& act_seq, const Buf& traj_q, const Buf& traj_qd,
                                   const Buf& status, const Buf& residual, int inverse_mode = BRAXG_INV_CHOLESKY) {
  braxg_dims d;
  int rc = braxg_model_dims(m, &d);
  if (rc) return last_error("braxg_model_dims", rc);
  int64_t n = -1;
  BRAXG_XLA_TRY(expect("q0", q0, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd0", qd0, {d.nv}, n));
  BRAXG_XLA_TRY(expect("act_seq", act_seq, {d.nu}, n, 1));
  BRAXG_XLA_TRY(expect("traj_q", traj_q, {d.nq}, n, 1));
  BRAXG_XLA_TRY(expect("traj_qd", traj_qd, {d.nv}, n, 1));
  BRAXG_XLA_TRY(expect("status", status, {}, n));
  const int64_t T = act_seq.dims[0];
  if (traj_q.dims[0] != T || traj_qd.dims[0] != T)
    return "act_seq, traj_q and traj_qd must share their leading (time) dimension";
  if (n > INT32_MAX || T > INT32_MAX || T < 1) return "the rollout needs 1 .. 2^31-1 steps and envs";
  BRAXG_XLA_TRY(expect_residual(m, n_frames, ckpt_every, q0, act_seq, residual, inverse_mode));
  braxg_options opt{};
  opt.inverse_mode = inverse_mode;
  rc = braxg_rollout_vjp_fwd(m, stream, static_cast<int>(n), static_cast<int>(T), n_frames, ckpt_every,
                             d.nu ? act_seq.f() : nullptr, q0.f(), qd0.f(), traj_q.f(), traj_qd.f(), residual.data,
                             static_cast<size_t>(residual.dims[0]), static_cast<int32_t*>(status.data), &opt);
  return rc ? last_error("braxg_rollout_vjp_fwd", rc) : "";
}

// jax.custom_vjp backward from that residual (only read: every segment is
// resident): cotangents q_bar [T, .., nq], qd_bar [T, .., nv] give act_bar
// [T, .., nu], q0_bar, qd0_bar.  `status` holds the forward's status (the
// handler aliases it) and gets the reverse's bits ORed in.
inline std::string rollout_vjp_bwd(const braxg_model* m, void* stream, int n_frames, int ckpt_every, const Buf& q0,
                                   const Buf& qd0, const Buf& act_seq, const Buf& residual, const Buf& q_bar,
                                   const Buf& qd_bar, const Buf& act_bar, const Buf& q0_bar, const Buf& qd0_bar,
                                   const Buf& status, int inverse_mode = BRAXG_INV_CHOLESKY) {
  braxg_dims d;
  int rc = braxg_model_dims(m, &d);
  if (rc) return last_error("braxg_model_dims", rc);
  int64_t n = -1;
  BRAXG_XLA_TRY(expect("q0", q0, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd0", qd0, {d.nv}, n));
  BRAXG_XLA_TRY(expect("act_seq", act_seq, {d.nu}, n, 1));
  BRAXG_XLA_TRY(expect("q_bar", q_bar, {d.nq}, n, 1));
  BRAXG_XLA_TRY(expect("qd_bar", qd_bar, {d.nv}, n, 1));
  BRAXG_XLA_TRY(expect("act_bar", act_bar, {d.nu}, n, 1));
  BRAXG_XLA_TRY(expect("q0_bar", q0_bar, {d.nq}, n));
  BRAXG_XLA_TRY(expect("qd0_bar", qd0_bar, {d.nv}, n));
  BRAXG_XLA_TRY(expect("status", status, {}, n));
  const int64_t T = act_seq.dims[0];
  if (q_bar.dims[0] != T || qd_bar.dims[0] != T || act_bar.dims[0] != T)
    return "act_seq, q_bar, qd_bar and act_bar must share their leading (time) dimension";
  if (n > INT32_MAX || T > INT32_MAX || T < 1) return "the rollout needs 1 .. 2^31-1 steps and envs";
  BRAXG_XLA_TRY(expect_residual(m, n_frames, ckpt_every, q0, act_seq, residual, inverse_mode));
  braxg_options opt{};
  opt.inverse_mode = inverse_mode;
  rc = braxg_rollout_vjp_bwd(m, stream, static_cast<int>(n), static_cast<int>(T), n_frames, ckpt_every,
                             d.nu ? act_seq.f() : nullptr, q0.f(), qd0.f(), q_bar.f(), qd_bar.f(),
                             d.nu ? act_bar.f() : nullptr, q0_bar.f(), qd0_bar.f(), residual.data,
                             static_cast<size_t>(residual.dims[0]), static_cast<int32_t*>(status.data), &opt);
  return rc ? last_error("braxg_rollout_vjp_bwd", rc) : "";
}

#undef BRAXG_XLA_TRY

}  // namespace braxg_xla
