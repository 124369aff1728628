// XLA FFI custom calls of the braxg kernels, for jax.jit(jax.vmap(...)) of
// the reference's pipeline functions (brax/generalized/pipeline.py:64-94
// under brax/envs/wrappers/training.py:66-72) and jax.grad through their
// scan (brax/training/agents/apg/train.py:188-198).  brax_gb300/jax_ops.py
// registers them (jax.ffi.register_ffi_target, platform "CUDA") and wraps the
// rollout in jax.custom_vjp.
//
// Each handler unpacks its buffers into braxg_xla::Buf and runs the shared
// core of xla_core.h (shape checks and the braxg C ABI calls).  This file is
// compiled only where jaxlib's FFI headers are present (build.py looks for
// them with jax.ffi.include_dir() or $BRAXG_XLA_INCLUDE) into libbraxg_xla.so,
// linked against libbraxg.so.
#include <cuda_runtime.h>

#include <cstdint>
#include <optional>
#include <string>

#include "xla/ffi/api/ffi.h"
#include "xla_core.h"

namespace ffi = xla::ffi;

namespace {

constexpr int kMaxRank = 8;

// A buffer's data pointer and a copy of its dimensions.
struct View {
  int64_t dims[kMaxRank];
  braxg_xla::Buf buf;
};

template <typename B>
View view(const B& b, void* data) {
  View v{};
  auto d = b.dimensions();
  const int r = static_cast<int>(d.size()) < kMaxRank ? static_cast<int>(d.size()) : kMaxRank;
  for (int i = 0; i < r; ++i) v.dims[i] = d[i];
  v.buf = braxg_xla::Buf{data, v.dims, r};
  return v;
}

template <ffi::DataType D>
View in(const ffi::Buffer<D>& b) {
  return view(b, const_cast<void*>(static_cast<const void*>(b.typed_data())));
}

template <ffi::DataType D>
View out(ffi::Result<ffi::Buffer<D>>& r) {
  return view(*r, static_cast<void*>(r->typed_data()));
}

ffi::Error to_error(const std::string& msg) {
  if (msg.empty()) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInvalidArgument, "braxg: " + msg);
}

const braxg_model* model_of(int64_t handle) { return reinterpret_cast<const braxg_model*>(handle); }

using F32 = ffi::Buffer<ffi::F32>;
using F32Out = ffi::Result<ffi::Buffer<ffi::F32>>;
using S32Out = ffi::Result<ffi::Buffer<ffi::S32>>;

ffi::Error StepImpl(cudaStream_t stream, int64_t model, int32_t n_frames, int32_t inverse_mode, F32 q, F32 qd,
                    F32 minv, F32 act, F32Out q_out, F32Out qd_out, F32Out minv_out, F32Out x_pos, F32Out x_rot,
                    F32Out xd_ang, F32Out xd_vel, F32Out qf_smooth, F32Out qf_constraint, F32Out qdd,
                    S32Out status) {
  View a = in(q), b = in(qd), c = in(minv), d = in(act);
  View o[11] = {out(q_out), out(qd_out), out(minv_out), out(x_pos), out(x_rot), out(xd_ang),
                out(xd_vel), out(qf_smooth), out(qf_constraint), out(qdd), out(status)};
  return to_error(braxg_xla::step(model_of(model), stream, n_frames, inverse_mode, a.buf, b.buf, c.buf, d.buf,
                                  o[0].buf, o[1].buf, o[2].buf, o[3].buf, o[4].buf, o[5].buf, o[6].buf, o[7].buf,
                                  o[8].buf, o[9].buf, o[10].buf));
}

ffi::Error RolloutImpl(cudaStream_t stream, ffi::ScratchAllocator scratch, int64_t model, int32_t n_frames,
                       int32_t inverse_mode, F32 q0, F32 qd0, F32 act_seq, F32Out traj_q, F32Out traj_qd,
                       S32Out status) {
  View a = in(q0), b = in(qd0), c = in(act_seq), tq = out(traj_q), tqd = out(traj_qd), st = out(status);
  const braxg_model* m = model_of(model);
  braxg_dims dm;
  if (braxg_model_dims(m, &dm)) return to_error(braxg_xla::last_error("braxg_model_dims", 1));
  const int64_t n = braxg_xla::envs_of(a.buf, {dm.nq});
  if (n < 0) return to_error("q0 has shape " + braxg_xla::dims_str(a.buf));
  const size_t floats = braxg_xla::rollout_scratch_floats(m, n);
  std::optional<void*> mem = scratch.Allocate(floats * sizeof(float) + 16, 16);
  if (!mem.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "braxg: rollout scratch");
  return to_error(braxg_xla::rollout(m, stream, n_frames, inverse_mode, a.buf, b.buf, c.buf, tq.buf, tqd.buf,
                                     st.buf, static_cast<float*>(*mem), floats));
}

ffi::Error RolloutVjpImpl(cudaStream_t stream, ffi::ScratchAllocator scratch, int64_t model, int32_t n_frames,
                          int32_t ckpt_every, int32_t inverse_mode, F32 q0, F32 qd0, F32 act_seq, F32 q_bar,
                          F32 qd_bar, F32Out act_bar, F32Out q0_bar, F32Out qd0_bar, S32Out status) {
  View a = in(q0), b = in(qd0), c = in(act_seq), d = in(q_bar), e = in(qd_bar);
  View ab = out(act_bar), qb = out(q0_bar), qdb = out(qd0_bar), st = out(status);
  const braxg_model* m = model_of(model);
  const size_t bytes = braxg_xla::rollout_vjp_workspace(m, n_frames, ckpt_every, a.buf, c.buf, inverse_mode);
  void* ws = nullptr;
  if (bytes > 0) {
    std::optional<void*> mem = scratch.Allocate(bytes, 256);
    if (mem.has_value()) ws = *mem;  // else: the library's fixed scratch (noalloc entry point)
  }
  return to_error(braxg_xla::rollout_vjp(m, stream, n_frames, ckpt_every, a.buf, b.buf, c.buf, d.buf, e.buf, ab.buf,
                                         qb.buf, qdb.buf, st.buf, ws, bytes, inverse_mode));
}

using U8 = ffi::Buffer<ffi::U8>;
using U8Out = ffi::Result<ffi::Buffer<ffi::U8>>;
using S32 = ffi::Buffer<ffi::S32>;

ffi::Error RolloutVjpFwdImpl(cudaStream_t stream, int64_t model, int32_t n_frames, int32_t ckpt_every,
                             int32_t inverse_mode, F32 q0, F32 qd0, F32 act_seq, F32Out traj_q, F32Out traj_qd,
                             S32Out status, U8Out residual) {
  View a = in(q0), b = in(qd0), c = in(act_seq);
  View tq = out(traj_q), tqd = out(traj_qd), st = out(status), rs = out(residual);
  return to_error(braxg_xla::rollout_vjp_fwd(model_of(model), stream, n_frames, ckpt_every, a.buf, b.buf, c.buf,
                                             tq.buf, tqd.buf, st.buf, rs.buf, inverse_mode));
}

// `status_in` is the forward's status; jax_ops aliases it with the `status`
// result (input_output_aliases), so both name one buffer.
ffi::Error RolloutVjpBwdImpl(cudaStream_t stream, int64_t model, int32_t n_frames, int32_t ckpt_every,
                             int32_t inverse_mode, F32 q0, F32 qd0, F32 act_seq, U8 residual, F32 q_bar,
                             F32 qd_bar, S32 status_in, F32Out act_bar, F32Out q0_bar, F32Out qd0_bar,
                             S32Out status) {
  (void)status_in;
  View a = in(q0), b = in(qd0), c = in(act_seq), r = in(residual), d = in(q_bar), e = in(qd_bar);
  View ab = out(act_bar), qb = out(q0_bar), qdb = out(qd0_bar), st = out(status);
  return to_error(braxg_xla::rollout_vjp_bwd(model_of(model), stream, n_frames, ckpt_every, a.buf, b.buf, c.buf,
                                             r.buf, d.buf, e.buf, ab.buf, qb.buf, qdb.buf, st.buf, inverse_mode));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(BraxgStepFfi, StepImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int32_t>("n_frames")
                                  .Attr<int32_t>("inverse_mode")
                                  .Arg<F32>()   // q
                                  .Arg<F32>()   // qd
                                  .Arg<F32>()   // mass_mx_inv
                                  .Arg<F32>()   // act
                                  .Ret<ffi::Buffer<ffi::F32>>()   // q
                                  .Ret<ffi::Buffer<ffi::F32>>()   // qd
                                  .Ret<ffi::Buffer<ffi::F32>>()   // mass_mx_inv
                                  .Ret<ffi::Buffer<ffi::F32>>()   // x.pos
                                  .Ret<ffi::Buffer<ffi::F32>>()   // x.rot
                                  .Ret<ffi::Buffer<ffi::F32>>()   // xd.ang
                                  .Ret<ffi::Buffer<ffi::F32>>()   // xd.vel
                                  .Ret<ffi::Buffer<ffi::F32>>()   // qf_smooth
                                  .Ret<ffi::Buffer<ffi::F32>>()   // qf_constraint
                                  .Ret<ffi::Buffer<ffi::F32>>()   // qdd
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status

XLA_FFI_DEFINE_HANDLER_SYMBOL(BraxgRolloutFfi, RolloutImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Attr<int64_t>("model")
                                  .Attr<int32_t>("n_frames")
                                  .Attr<int32_t>("inverse_mode")
                                  .Arg<F32>()   // q0
                                  .Arg<F32>()   // qd0
                                  .Arg<F32>()   // act_seq [T, .., nu]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // traj_q [T, .., nq]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // traj_qd [T, .., nv]
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status

XLA_FFI_DEFINE_HANDLER_SYMBOL(BraxgRolloutVjpFfi, RolloutVjpImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Attr<int64_t>("model")
                                  .Attr<int32_t>("n_frames")
                                  .Attr<int32_t>("ckpt_every")
                                  .Attr<int32_t>("inverse_mode")
                                  .Arg<F32>()   // q0
                                  .Arg<F32>()   // qd0
                                  .Arg<F32>()   // act_seq
                                  .Arg<F32>()   // q_bar [T, .., nq]
                                  .Arg<F32>()   // qd_bar [T, .., nv]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // act_bar [T, .., nu]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // q0_bar
                                  .Ret<ffi::Buffer<ffi::F32>>()   // qd0_bar
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status

XLA_FFI_DEFINE_HANDLER_SYMBOL(BraxgRolloutVjpFwdFfi, RolloutVjpFwdImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int32_t>("n_frames")
                                  .Attr<int32_t>("ckpt_every")
                                  .Attr<int32_t>("inverse_mode")
                                  .Arg<F32>()   // q0
                                  .Arg<F32>()   // qd0
                                  .Arg<F32>()   // act_seq [T, .., nu]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // traj_q [T, .., nq]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // traj_qd [T, .., nv]
                                  .Ret<ffi::Buffer<ffi::S32>>()   // status
                                  .Ret<ffi::Buffer<ffi::U8>>());  // residual [bytes]

XLA_FFI_DEFINE_HANDLER_SYMBOL(BraxgRolloutVjpBwdFfi, RolloutVjpBwdImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int32_t>("n_frames")
                                  .Attr<int32_t>("ckpt_every")
                                  .Attr<int32_t>("inverse_mode")
                                  .Arg<F32>()   // q0
                                  .Arg<F32>()   // qd0
                                  .Arg<F32>()   // act_seq
                                  .Arg<U8>()    // residual
                                  .Arg<F32>()   // q_bar [T, .., nq]
                                  .Arg<F32>()   // qd_bar [T, .., nv]
                                  .Arg<S32>()   // the forward's status (aliased with the status result)
                                  .Ret<ffi::Buffer<ffi::F32>>()   // act_bar [T, .., nu]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // q0_bar
                                  .Ret<ffi::Buffer<ffi::F32>>()   // qd0_bar
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status
