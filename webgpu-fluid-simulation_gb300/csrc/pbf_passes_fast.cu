// pbf_passes_fast.cu — the float passes with FMA contraction (production).
#define PBF_NS fast
#define PBF_FAST_MATH 1
#include "pbf_passes.cuh"
