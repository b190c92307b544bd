// Kernel-variant autotuner.  A tunable launch (a GEMM of a given shape, type
// and transposition) is identified by a key; the first time a key is met
// outside stream capture, every variant runs on scratch output buffers, is
// timed with CUDA events on the context's stream, and the fastest is kept in
// a process-wide table (optionally appended to the file named by
// IA_TUNE_FILE and read back from it by later processes).  IA_TUNE=0 turns
// tuning off (variant 0 everywhere).  Variants of one kernel differ only in
// the mapping of outputs to threads, never in the order of the sums, so the
// choice does not change results.
#pragma once
#include <functional>
#include "ia_internal.h"

namespace ia {

struct TuneKey {
    int kernel;      // TuneKernel
    int device;
    int v[8];        // shape / op parameters
};

enum TuneKernel {
    TK_GEMM_Z = 1,
    TK_GEMM_C = 2,
    TK_DFGEMM = 3,
    TK_RGEMM_D = 4,
    TK_RGEMM_S = 5,
    TK_RDFGEMM = 6,
    TK_DFGEMM4 = 7
};

// Variant for key: the table entry, or (when absent) the result of timing
// run(variant) for variant in [0, nvar) -- run must launch on scratch outputs --
// or 0 when tuning is off, the stream is capturing or the call may not
// allocate (ctx->no_tune).
int tune_select(ia_context *ctx, TuneKey key, int nvar, const std::function<int(int)> &run);

// Scratch for tuning runs: a stream-ordered allocation holding a copy of the
// output region [C, C + bytes) so beta != 0 launches read the same values.
struct TuneScratch {
    ia_context *ctx;
    void *p = nullptr;
    int init(const void *src, size_t bytes);
    ~TuneScratch();
};

}  // namespace ia
