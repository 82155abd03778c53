// pbf_passes_fast.cu — the float passes with FMA contraction (production).
#define PBF_NS fast
#include "pbf_passes.cuh"
