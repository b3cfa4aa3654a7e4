// The single-set build's kernels once more, compiled with the widest exact
// tier (QDTG_WIDE_EXACT 1) and with every predicate call counted
// (QDTG_COUNT_CALLS 1) into qdtg::wide: the engine runs a call again with
// these when a predicate of the default kernels (qdtg::narrow) needed that
// tier, which only coordinates spanning more than 95 bits inside one
// predicate do, and runs them from the start when the call counts.
#define QDTG_WIDE_EXACT 1
#define QDTG_COUNT_CALLS 1
#define QDTG_BUILD_VARIANT wide
#include "k_build.cu"
