// The batch build's predicate kernels once more, compiled with the widest
// exact tier (QDTG_WIDE_EXACT 1) into qdtg::wide: the batch engine runs the
// stages after its host synchronisation again with these when a predicate
// of the default kernels (qdtg::narrow) needed that tier, which only
// coordinates spanning more than 95 bits inside one predicate do.
#define QDTG_WIDE_EXACT 1
#define QDTG_BUILD_VARIANT wide
#include "batch_build.cu"
