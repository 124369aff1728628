// Host-side test of the checked build's scratch checks: for the model
// dimensions on the command line (nl nq nv nu ncon nlim ns_iters fluid per
// model) it lays out the per-env arena with the kernels' make_layout and
// checks every stage's declared scratch use (the ScratchUse functions the
// stages pass to bx_scratch) with scratch_use_ok, the function behind the
// BRAXG_ENV_BOUNDS bit:
//   1. on the real layouts (cache and no-cache overflow placements) every
//      use fits, for every active row count;
//   2. on a deliberately undersized arena (scratch cut short by 8 words, or
//      the mass matrix moved onto the Jacobian stage's region) the check
//      fails, i.e. the checked kernel would set the bit.
// Prints "ok <checks>" and exits 0 when both hold.
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "braxg_step.cuh"

using namespace braxg;

static int g_checks = 0;
#define CHECK(cond)                                                          \
  do {                                                                       \
    ++g_checks;                                                              \
    if (!(cond)) {                                                           \
      std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      std::exit(1);                                                          \
    }                                                                        \
  } while (0)

// every stage's declared use on layout L; returns how many fail (and, in
// *max_end, the furthest word any of them reaches)
static int failures(const Layout& L, int nl, int nv, int nu, int ncon, int m, bool fluid, int* max_end = nullptr) {
  std::vector<ScratchUse> uses = {scratch_fk(L, nl, nv),         scratch_crba(L, nl, nv),
                                  scratch_inverse(L, nv, true, false),
                                  scratch_inverse(L, nv, false, nv <= 16),
                                  scratch_jacobian(L, ncon),       scratch_smooth(L, nl, nu, fluid),
                                  scratch_outputs(L, m, ncon)};
  for (int nrow = 1; nrow <= (m < kMaxExplicitRows ? m : kMaxExplicitRows); ++nrow)
    uses.push_back(scratch_pg_explicit(L, nrow));
  if (m > kMaxExplicitRows) uses.push_back(scratch_pg_implicit(L, m, nv));
  if (L.M < L.scr) uses.push_back(scratch_integrate(L, nv));  // models whose integrator owns M
  int bad = 0, far = 0;
  for (const ScratchUse& u : uses) {
    bad += scratch_use_ok(L, u, nv) ? 0 : 1;
    // a region that must keep the overflow rows reaches them at most
    far = std::max(far, u.keep_ovf && !L.ovf_g ? u.end + (L.scr + L.scr_words - L.jovf) : u.end);
  }
  if (max_end) *max_end = far;
  return bad;
}

int main(int argc, char** argv) {
  if ((argc - 1) % 8 != 0 || argc < 9) {
    std::fprintf(stderr, "usage: layout_check (nl nq nv nu ncon nlim ns_iters fluid)...\n");
    return 2;
  }
  int models = 0;
  for (int a = 1; a + 7 < argc; a += 8) {
    const int nl = atoi(argv[a]), nq = atoi(argv[a + 1]), nv = atoi(argv[a + 2]), nu = atoi(argv[a + 3]);
    const int ncon = atoi(argv[a + 4]), nlim = atoi(argv[a + 5]), ns = atoi(argv[a + 6]), fl = atoi(argv[a + 7]);
    const int m = 4 * ncon + nlim;
    for (int ovf_g = 0; ovf_g < 2; ++ovf_g) {
      Layout L = make_layout(nl, nq, nv, nu, ncon, nlim, ns, fl, ovf_g);
      CHECK(L.mrows == m);
      CHECK(L.canary + kCanaryWords == L.total);
      int far = 0;
      CHECK(failures(L, nl, nv, nu, ncon, m, fl != 0, &far) == 0);
      CHECK(far <= L.scr + L.scr_words);
      // undersized: scratch one word short of its largest user (the overflow
      // rows keeping their place at the scratch end)
      Layout S = L;
      const int cut = L.scr + L.scr_words - (far - 1);
      S.scr_words -= cut;
      if (!ovf_g) S.jovf -= cut;
      CHECK(failures(S, nl, nv, nu, ncon, m, fl != 0) > 0);
      // the mass matrix placed at the start of scratch, under the Jacobian stage's contacts
      if (ncon > 0 && ns != 0) {
        Layout C = L;
        C.M = C.scr;
        CHECK(!scratch_use_ok(C, scratch_jacobian(C, ncon), nv));
      }
      // the overflow rows kept by the constraint stage: an implicit solve's
      // region reaching into them
      if (m > kMaxExplicitRows && !ovf_g) {
        ScratchUse u = scratch_pg_implicit(L, m, nv);
        u.end = L.jovf + 1;
        CHECK(!scratch_use_ok(L, u, nv));
      }
    }
    ++models;
  }
  std::printf("ok %d checks over %d models\n", g_checks, models);
  return 0;
}
