// Bounds checks of the checked build (compiled with -DBRAXG_CHECK; the
// default build compiles every check to nothing).
//
// What is checked, per env:
// * scratch carve-outs: every stage that lays its temporaries into the
//   arena's scratch region checks the end of its last region against the end
//   of scratch, against the start of the overflow Jacobian rows when the
//   stage must keep them, and against the mass matrix when it lives in
//   scratch (scratch_ok below, shared with the host-side test);
// * Jacobian row indices (Ws::jrow) against the model's row count;
// * the 16-byte alignment of float4 copies and matvec operands;
// * canary words after every env's arena, verified at the entry of every
//   stage, so that a write past any region of the arena is caught.
// A failed check sets a bit in the env's misc[13] word; every later stage of
// the env returns at once (the CTA barriers are still taken), and the env's
// status gets BRAXG_ENV_BOUNDS.  Nothing traps.
#pragma once

namespace braxg {

#ifdef BRAXG_CHECK
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

// words after each arena holding the canary (checked build only)
constexpr int kCanaryWords = kChecked ? 4 : 0;
constexpr unsigned kCanary = 0x7fc0de5au;  // a NaN pattern no stage writes

// bits of misc[13]
enum BoundsBits : unsigned {
  kBoundsScratch = 1u,  // a scratch region past its end or over live data
  kBoundsRow = 2u,      // a Jacobian row index outside the model's rows
  kBoundsAlign = 4u,    // a float4 access not 16-byte aligned
  kBoundsCanary = 8u,   // the canary after the arena was overwritten
};

// Whether a scratch region ending at word `end` (arena offset) fits: inside
// the scratch region, before the overflow Jacobian rows when the stage must
// keep them (they live at the scratch end unless they are in the cache), and
// not over the mass matrix when it lives in scratch and must be kept
// ([m_lo, m_hi) arena offsets, empty when m_lo >= m_hi).  `start` is the
// region's first word.
__host__ __device__ inline bool scratch_ok(int scr, int scr_words, int jovf, bool ovf_in_scratch, bool keep_ovf,
                                           int start, int end, int m_lo, int m_hi) {
  if (start < scr || end > scr + scr_words) return false;
  if (keep_ovf && ovf_in_scratch && end > jovf) return false;
  if (m_lo < m_hi && start < m_hi && end > m_lo) return false;
  return true;
}

}  // namespace braxg
