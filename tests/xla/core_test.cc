// Host-only test of the XLA handler core (brax_gb300/csrc/xla/xla_core.h):
// compiled with a stub of the braxg C calls that records what it receives,
// it checks the shape rules (jax.vmap batch axes, time axes), the error
// messages, and the pointers, env counts and options each call forwards.
// Prints "ok <n>" and exits 0 when every case passes.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "xla_core.h"

// ---- stub of the braxg C ABI ------------------------------------------------
struct braxg_model {
  braxg_dims dims;
};

struct Call {
  std::string name;
  int n_env = -1, n_steps = -1, n_frames = -1, ckpt = -1, inverse_mode = -1;
  const void* p[8] = {};
  void* ws = nullptr;
  size_t ws_bytes = 0;
};
static std::vector<Call> g_calls;
static size_t g_ws_bytes = 1000;

extern "C" {
int braxg_model_dims(const braxg_model* m, braxg_dims* out) {
  *out = m->dims;
  return 0;
}
const char* braxg_last_error(void) { return "stub"; }
int braxg_init(const braxg_model*, void*, int n_env, const float* q, const float* qd, braxg_state* out,
               const braxg_options* opt) {
  Call c;
  c.name = "init";
  c.n_env = n_env;
  c.inverse_mode = opt ? opt->inverse_mode : -1;
  c.p[0] = q;
  c.p[1] = qd;
  c.p[2] = out->mass_mx_inv;
  g_calls.push_back(c);
  return 0;
}
int braxg_step(const braxg_model*, void*, int n_env, int n_frames, const float* act, const braxg_state* in,
               braxg_state* out, const braxg_options* opt) {
  Call c;
  c.name = "step";
  c.n_env = n_env;
  c.n_frames = n_frames;
  c.inverse_mode = opt->inverse_mode;
  c.p[0] = in->q;
  c.p[1] = in->qd;
  c.p[2] = in->mass_mx_inv;
  c.p[3] = act;
  c.p[4] = out->q;
  c.p[5] = out->x_rot;
  c.p[6] = out->status;
  c.p[7] = out->qdd;
  g_calls.push_back(c);
  return 0;
}
int braxg_rollout(const braxg_model*, void*, int n_env, int n_steps, int n_frames, const float* act_seq,
                  const braxg_state* in, braxg_state* out, float* traj_q, float* traj_qd, const braxg_options* opt) {
  Call c;
  c.name = "rollout";
  c.n_env = n_env;
  c.n_steps = n_steps;
  c.n_frames = n_frames;
  c.inverse_mode = opt->inverse_mode;
  c.p[0] = in->q;
  c.p[1] = in->mass_mx_inv;
  c.p[2] = act_seq;
  c.p[3] = traj_q;
  c.p[4] = traj_qd;
  c.p[5] = out->mass_mx_inv;
  g_calls.push_back(c);
  return 0;
}
int braxg_rollout_vjp_workspace(const braxg_model*, int, int, int, int, size_t* bytes) {
  *bytes = g_ws_bytes;
  return 0;
}
int braxg_rollout_vjp(const braxg_model*, void*, int n_env, int n_steps, int n_frames, int ckpt_every,
                      const float* act_seq, const float* q0, const float*, const float* q_bar, const float*,
                      float* act_bar, float* q0_bar, float*, float*, float*, void* workspace, size_t workspace_bytes,
                      int32_t*, const braxg_options* opt) {
  Call c;
  c.name = "vjp";
  c.n_env = n_env;
  c.n_steps = n_steps;
  c.n_frames = n_frames;
  c.ckpt = ckpt_every;
  c.inverse_mode = opt->inverse_mode;
  c.p[0] = act_seq;
  c.p[1] = q0;
  c.p[2] = q_bar;
  c.p[3] = act_bar;
  c.p[4] = q0_bar;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  g_calls.push_back(c);
  return 0;
}
int braxg_rollout_vjp_workspace_resident(const braxg_model*, int, int, int, int, int resident, size_t* bytes) {
  *bytes = resident <= 0 ? 2 * g_ws_bytes : g_ws_bytes;  // every segment resident: the larger workspace
  return 0;
}
// Newton-Schulz mode adds the per-frame records: 500 bytes more in the stub
int braxg_rollout_vjp_workspace_mode(const braxg_model* m, int n_env, int n_steps, int n_frames, int ckpt_every,
                                     int resident, int inverse_mode, size_t* bytes) {
  braxg_rollout_vjp_workspace_resident(m, n_env, n_steps, n_frames, ckpt_every, resident, bytes);
  if (inverse_mode == BRAXG_INV_NEWTON_SCHULZ) *bytes += 500;
  return 0;
}
int braxg_rollout_vjp_fwd(const braxg_model*, void*, int n_env, int n_steps, int n_frames, int ckpt_every,
                          const float* act_seq, const float* q0, const float*, float* traj_q, float* traj_qd,
                          void* workspace, size_t workspace_bytes, int32_t* status, const braxg_options* opt) {
  Call c;
  c.name = "vjp_fwd";
  c.n_env = n_env;
  c.n_steps = n_steps;
  c.n_frames = n_frames;
  c.ckpt = ckpt_every;
  c.inverse_mode = opt->inverse_mode;
  c.p[0] = act_seq;
  c.p[1] = q0;
  c.p[2] = traj_q;
  c.p[3] = traj_qd;
  c.p[4] = status;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  g_calls.push_back(c);
  return 0;
}
int braxg_rollout_vjp_bwd(const braxg_model*, void*, int n_env, int n_steps, int n_frames, int ckpt_every,
                          const float* act_seq, const float* q0, const float*, const float* q_bar, const float*,
                          float* act_bar, float* q0_bar, float*, void* workspace, size_t workspace_bytes,
                          int32_t* status, const braxg_options* opt) {
  Call c;
  c.name = "vjp_bwd";
  c.n_env = n_env;
  c.n_steps = n_steps;
  c.n_frames = n_frames;
  c.ckpt = ckpt_every;
  c.inverse_mode = opt->inverse_mode;
  c.p[0] = act_seq;
  c.p[1] = q0;
  c.p[2] = q_bar;
  c.p[3] = act_bar;
  c.p[4] = q0_bar;
  c.p[5] = status;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  g_calls.push_back(c);
  return 0;
}
int braxg_rollout_vjp_noalloc(const braxg_model*, void*, int n_env, int n_steps, int, int, const float*,
                              const float*, const float*, const float*, const float*, float*, float*, float*, float*,
                              float*, int32_t*, const braxg_options*) {
  Call c;
  c.name = "vjp_noalloc";
  c.n_env = n_env;
  c.n_steps = n_steps;
  g_calls.push_back(c);
  return 0;
}
}

// ---- test helpers ------------------------------------------------------------
static int g_checks = 0;
#define CHECK(cond)                                                         \
  do {                                                                      \
    ++g_checks;                                                             \
    if (!(cond)) {                                                          \
      std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      std::exit(1);                                                         \
    }                                                                       \
  } while (0)

// An owned buffer of the given dimensions.
struct Arr {
  std::vector<int64_t> dims;
  std::vector<float> data;
  explicit Arr(std::vector<int64_t> d) : dims(d) {
    size_t n = 1;
    for (int64_t x : d) n *= static_cast<size_t>(x);
    data.assign(n > 0 ? n : 1, 0.f);
  }
  braxg_xla::Buf buf() { return braxg_xla::Buf{data.data(), dims.data(), static_cast<int>(dims.size())}; }
};

static bool contains(const std::string& s, const char* part) { return s.find(part) != std::string::npos; }

int main() {
  braxg_model m{};
  m.dims = braxg_dims{9, 15, 14, 8, 17, 0, 68};  // the quadruped
  const int nl = 9, nq = 15, nv = 14, nu = 8;

  // ---- step: batched [n, ...] -------------------------------------------------
  {
    const int n = 6;
    Arr q({n, nq}), qd({n, nv}), mi({n, nv, nv}), act({n, nu});
    Arr qo({n, nq}), qdo({n, nv}), mio({n, nv, nv}), xp({n, nl, 3}), xr({n, nl, 4}), xa({n, nl, 3}),
        xv({n, nl, 3}), qfs({n, nv}), qfc({n, nv}), qdd({n, nv}), st({n});
    g_calls.clear();
    std::string e = braxg_xla::step(&m, nullptr, 5, BRAXG_INV_CHOLESKY, q.buf(), qd.buf(), mi.buf(), act.buf(),
                                    qo.buf(), qdo.buf(), mio.buf(), xp.buf(), xr.buf(), xa.buf(), xv.buf(),
                                    qfs.buf(), qfc.buf(), qdd.buf(), st.buf());
    CHECK(e.empty());
    CHECK(g_calls.size() == 1 && g_calls[0].name == "step");
    const Call& c = g_calls[0];
    CHECK(c.n_env == n && c.n_frames == 5 && c.inverse_mode == BRAXG_INV_CHOLESKY);
    CHECK(c.p[0] == q.data.data() && c.p[1] == qd.data.data() && c.p[2] == mi.data.data());
    CHECK(c.p[3] == act.data.data() && c.p[4] == qo.data.data() && c.p[5] == xr.data.data());
    CHECK(c.p[6] == st.data.data() && c.p[7] == qdd.data.data());

    // nested vmap axes [2, 3, ...] are one batch of 6 envs
    Arr q2({2, 3, nq}), qd2({2, 3, nv}), mi2({2, 3, nv, nv}), act2({2, 3, nu}), st2({2, 3});
    g_calls.clear();
    e = braxg_xla::step(&m, nullptr, 1, BRAXG_INV_NEWTON_SCHULZ, q2.buf(), qd2.buf(), mi2.buf(), act2.buf(),
                        qo.buf(), qdo.buf(), mio.buf(), xp.buf(), xr.buf(), xa.buf(), xv.buf(), qfs.buf(),
                        qfc.buf(), qdd.buf(), st2.buf());
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].n_env == 6);

    // an unbatched call (the reference's per-env signature) is one env
    Arr q1({nq}), qd1({nv}), mi1({nv, nv}), act1({nu}), qo1({nq}), qdo1({nv}), mio1({nv, nv}), xp1({nl, 3}),
        xr1({nl, 4}), xa1({nl, 3}), xv1({nl, 3}), f1({nv}), f2({nv}), f3({nv}), st1({});
    g_calls.clear();
    e = braxg_xla::step(&m, nullptr, 1, 0, q1.buf(), qd1.buf(), mi1.buf(), act1.buf(), qo1.buf(), qdo1.buf(),
                        mio1.buf(), xp1.buf(), xr1.buf(), xa1.buf(), xv1.buf(), f1.buf(), f2.buf(), f3.buf(),
                        st1.buf());
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].n_env == 1);

    // wrong trailing shape: refused before any call, the message names the argument
    Arr bad({n, nv + 1});
    g_calls.clear();
    e = braxg_xla::step(&m, nullptr, 1, 0, q.buf(), bad.buf(), mi.buf(), act.buf(), qo.buf(), qdo.buf(), mio.buf(),
                        xp.buf(), xr.buf(), xa.buf(), xv.buf(), qfs.buf(), qfc.buf(), qdd.buf(), st.buf());
    CHECK(contains(e, "qd has shape [6, 15]") && g_calls.empty());
    // batch sizes that disagree
    Arr act7({7, nu});
    e = braxg_xla::step(&m, nullptr, 1, 0, q.buf(), qd.buf(), mi.buf(), act7.buf(), qo.buf(), qdo.buf(), mio.buf(),
                        xp.buf(), xr.buf(), xa.buf(), xv.buf(), qfs.buf(), qfc.buf(), qdd.buf(), st.buf());
    CHECK(contains(e, "act holds 7 envs, expected 6") && g_calls.empty());
  }

  // ---- rollout: [T, n, ...] sequences ------------------------------------------
  {
    const int n = 4, T = 3;
    Arr q0({n, nq}), qd0({n, nv}), a({T, n, nu}), tq({T, n, nq}), tqd({T, n, nv}), st({n});
    std::vector<float> scr(braxg_xla::rollout_scratch_floats(&m, n));
    CHECK(scr.size() == static_cast<size_t>(2 * n * nv * nv));
    g_calls.clear();
    std::string e = braxg_xla::rollout(&m, nullptr, 5, BRAXG_INV_NEWTON_SCHULZ, q0.buf(), qd0.buf(), a.buf(),
                                       tq.buf(), tqd.buf(), st.buf(), scr.data(), scr.size());
    CHECK(e.empty());
    CHECK(g_calls.size() == 2 && g_calls[0].name == "init" && g_calls[1].name == "rollout");
    CHECK(g_calls[0].n_env == n && g_calls[0].p[2] == scr.data());
    const Call& r = g_calls[1];
    CHECK(r.n_env == n && r.n_steps == T && r.n_frames == 5 && r.inverse_mode == BRAXG_INV_NEWTON_SCHULZ);
    CHECK(r.p[0] == q0.data.data() && r.p[1] == scr.data() && r.p[2] == a.data.data());
    CHECK(r.p[3] == tq.data.data() && r.p[4] == tqd.data.data() && r.p[5] == scr.data() + n * nv * nv);
    // time axes that disagree
    Arr tq2({T + 1, n, nq});
    e = braxg_xla::rollout(&m, nullptr, 5, 0, q0.buf(), qd0.buf(), a.buf(), tq2.buf(), tqd.buf(), st.buf(),
                           scr.data(), scr.size());
    CHECK(contains(e, "leading (time) dimension"));
    // too little scratch
    e = braxg_xla::rollout(&m, nullptr, 5, 0, q0.buf(), qd0.buf(), a.buf(), tq.buf(), tqd.buf(), st.buf(),
                           scr.data(), scr.size() - 1);
    CHECK(contains(e, "scratch too small"));
  }

  // ---- rollout_vjp: workspace, or the fixed scratch without one ------------------
  {
    const int n = 4, T = 6;
    Arr q0({n, nq}), qd0({n, nv}), a({T, n, nu}), qb({T, n, nq}), qdb({T, n, nv}), ab({T, n, nu}), q0b({n, nq}),
        qd0b({n, nv}), st({n});
    g_ws_bytes = 12345;
    const size_t bytes = braxg_xla::rollout_vjp_workspace(&m, 5, 2, q0.buf(), a.buf());
    CHECK(bytes == 12345);
    std::vector<char> ws(bytes);
    g_calls.clear();
    std::string e = braxg_xla::rollout_vjp(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), qb.buf(), qdb.buf(),
                                           ab.buf(), q0b.buf(), qd0b.buf(), st.buf(), ws.data(), bytes);
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].name == "vjp");
    const Call& c = g_calls[0];
    CHECK(c.n_env == n && c.n_steps == T && c.n_frames == 5 && c.ckpt == 2);
    CHECK(c.inverse_mode == BRAXG_INV_CHOLESKY);  // gradients use the exact inverse
    CHECK(c.p[0] == a.data.data() && c.p[1] == q0.data.data() && c.p[2] == qb.data.data());
    CHECK(c.p[3] == ab.data.data() && c.p[4] == q0b.data.data());
    CHECK(c.ws == ws.data() && c.ws_bytes == bytes);
    g_calls.clear();
    e = braxg_xla::rollout_vjp(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), qb.buf(), qdb.buf(), ab.buf(),
                               q0b.buf(), qd0b.buf(), st.buf(), nullptr, 0);
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].name == "vjp_noalloc" && g_calls[0].n_env == n);
    Arr qdb_bad({T, n, nv - 1});
    e = braxg_xla::rollout_vjp(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), qb.buf(), qdb_bad.buf(), ab.buf(),
                               q0b.buf(), qd0b.buf(), st.buf(), ws.data(), bytes);
    CHECK(contains(e, "qd_bar has shape"));
    // the reference's inverse mode: its workspace and the option reach the call
    const size_t ns_bytes = braxg_xla::rollout_vjp_workspace(&m, 5, 2, q0.buf(), a.buf(), BRAXG_INV_NEWTON_SCHULZ);
    CHECK(ns_bytes == 12345 + 500);
    std::vector<char> ws_ns(ns_bytes);
    g_calls.clear();
    e = braxg_xla::rollout_vjp(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), qb.buf(), qdb.buf(), ab.buf(),
                               q0b.buf(), qd0b.buf(), st.buf(), ws_ns.data(), ns_bytes, BRAXG_INV_NEWTON_SCHULZ);
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].inverse_mode == BRAXG_INV_NEWTON_SCHULZ);
    CHECK(g_calls[0].ws_bytes == ns_bytes);
  }
  // ---- rollout_vjp_fwd / rollout_vjp_bwd: the custom_vjp halves and their residual ----
  {
    const int n = 4, T = 6;
    Arr q0({n, nq}), qd0({n, nv}), a({T, n, nu}), tq({T, n, nq}), tqd({T, n, nv}), st({n}), qb({T, n, nq}),
        qdb({T, n, nv}), ab({T, n, nu}), q0b({n, nq}), qd0b({n, nv});
    g_ws_bytes = 1000;
    const size_t need = braxg_xla::rollout_vjp_residual_bytes(&m, 5, 2, q0.buf(), a.buf());
    CHECK(need == 2000);  // the workspace with every segment resident
    std::vector<int64_t> rdims = {static_cast<int64_t>(need)};
    std::vector<unsigned char> res(need);
    braxg_xla::Buf rbuf{res.data(), rdims.data(), 1};
    g_calls.clear();
    std::string e = braxg_xla::rollout_vjp_fwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), tq.buf(), tqd.buf(),
                                               st.buf(), rbuf);
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].name == "vjp_fwd");
    const Call& f = g_calls[0];
    CHECK(f.n_env == n && f.n_steps == T && f.n_frames == 5 && f.ckpt == 2 && f.inverse_mode == BRAXG_INV_CHOLESKY);
    CHECK(f.p[0] == a.data.data() && f.p[1] == q0.data.data() && f.p[2] == tq.data.data());
    CHECK(f.p[3] == tqd.data.data() && f.p[4] == st.data.data());
    CHECK(f.ws == res.data() && f.ws_bytes == need);
    g_calls.clear();
    e = braxg_xla::rollout_vjp_bwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), rbuf, qb.buf(), qdb.buf(),
                                   ab.buf(), q0b.buf(), qd0b.buf(), st.buf());
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].name == "vjp_bwd");
    const Call& b = g_calls[0];
    CHECK(b.n_env == n && b.n_steps == T && b.ckpt == 2 && b.inverse_mode == BRAXG_INV_CHOLESKY);
    CHECK(b.p[0] == a.data.data() && b.p[1] == q0.data.data() && b.p[2] == qb.data.data());
    CHECK(b.p[3] == ab.data.data() && b.p[4] == q0b.data.data() && b.p[5] == st.data.data());
    CHECK(b.ws == res.data() && b.ws_bytes == need);
    // a residual smaller than the resident workspace is refused before any call
    std::vector<int64_t> small = {static_cast<int64_t>(need - 1)};
    braxg_xla::Buf rsmall{res.data(), small.data(), 1};
    g_calls.clear();
    e = braxg_xla::rollout_vjp_fwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), tq.buf(), tqd.buf(), st.buf(),
                                   rsmall);
    CHECK(contains(e, "residual has shape") && g_calls.empty());
    e = braxg_xla::rollout_vjp_bwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), rsmall, qb.buf(), qdb.buf(),
                                   ab.buf(), q0b.buf(), qd0b.buf(), st.buf());
    CHECK(contains(e, "residual has shape") && g_calls.empty());
    // the trajectory's time axis must match the actions'
    Arr tq_bad({T - 1, n, nq});
    e = braxg_xla::rollout_vjp_fwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), tq_bad.buf(), tqd.buf(),
                                   st.buf(), rbuf);
    CHECK(contains(e, "leading (time) dimension") && g_calls.empty());
    // Newton-Schulz mode: its residual holds the per-frame records too, and
    // the Cholesky-sized residual is refused for it
    const size_t need_ns =
        braxg_xla::rollout_vjp_residual_bytes(&m, 5, 2, q0.buf(), a.buf(), BRAXG_INV_NEWTON_SCHULZ);
    CHECK(need_ns == 2500);
    g_calls.clear();
    e = braxg_xla::rollout_vjp_fwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), tq.buf(), tqd.buf(), st.buf(),
                                   rbuf, BRAXG_INV_NEWTON_SCHULZ);
    CHECK(contains(e, "residual has shape") && g_calls.empty());
    std::vector<int64_t> nsdims = {static_cast<int64_t>(need_ns)};
    std::vector<unsigned char> res_ns(need_ns);
    braxg_xla::Buf rns{res_ns.data(), nsdims.data(), 1};
    e = braxg_xla::rollout_vjp_fwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), tq.buf(), tqd.buf(), st.buf(),
                                   rns, BRAXG_INV_NEWTON_SCHULZ);
    CHECK(e.empty() && g_calls.size() == 1 && g_calls[0].inverse_mode == BRAXG_INV_NEWTON_SCHULZ);
    e = braxg_xla::rollout_vjp_bwd(&m, nullptr, 5, 2, q0.buf(), qd0.buf(), a.buf(), rns, qb.buf(), qdb.buf(),
                                   ab.buf(), q0b.buf(), qd0b.buf(), st.buf(), BRAXG_INV_NEWTON_SCHULZ);
    CHECK(e.empty() && g_calls.size() == 2 && g_calls[1].inverse_mode == BRAXG_INV_NEWTON_SCHULZ);
    CHECK(g_calls[1].ws_bytes == need_ns);
  }
  std::printf("ok %d\n", g_checks);
  return 0;
}
