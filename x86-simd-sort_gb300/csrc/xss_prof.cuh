// xss_prof.cuh -- kernel kinds for launch counting / event timing (xss_prof.cu).
#pragma once
#include <cuda_runtime.h>

namespace xss {

enum ProfKind : int {
    PK_HIST = 0,       // up-front digit histogram (+ pass plan)
    PK_ONESWEEP = 1,   // one LSD radix pass
    PK_FIXUP = 2,      // copy-back / canonicalise / iota after the passes
    PK_SMALL = 3,      // one-CTA sort of a small array
    PK_SEL_HIST = 4,   // radix-select digit histogram
    PK_SEL_FIND = 5,   // radix-select bucket search
    PK_SEL_COLLECT = 6,// partition: find misplaced elements
    PK_SEL_PLACE = 7,  // partition: move them into place
    PK_SEG_SMALL = 8,  // segmented sort: many small segments per launch
    PK_SEG_BLOCK = 9,  // segmented sort: one CTA per medium segment
    PK_SEG_MISC = 10,  // segmented sort: binning / bookkeeping
    PK_OBJECT = 11,    // record sort: key extraction / record gather
    PK_MERGE = 12,     // chunked sort of a very large array: merge of sorted runs
    PK_COUNT16 = 13,   // 16-bit keys-only sort by counting: counts, scan, expansion
    PK_COUNT = 14
};

void prof_begin(cudaStream_t s, int kind);
void prof_end(cudaStream_t s, int kind);
// Snapshot of the per-kind launch counters (PK_COUNT entries), and a bulk
// add -- used to count kernels that run inside a replayed CUDA graph.
void prof_snapshot(unsigned long long *out);
void prof_add(const unsigned long long *counts);
void prof_sub(const unsigned long long *counts);

}  // namespace xss
