// pbf_passes_exact.cu — the float passes compiled with -fmad=false: no
// multiply-add contraction, so every result is bit-identical with the CPU
// restatement of the reference (which is compiled with -ffp-contract=off).
#define PBF_NS exact
#include "pbf_passes.cuh"
