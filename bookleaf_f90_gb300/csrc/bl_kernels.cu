// bl_kernels.cu -- the translation unit holding every hot-path kernel.
// Compiled twice with -DBL_NS=fast (--fmad=true) and -DBL_NS=exact
// (--fmad=false); see bl_kernels.h.
#ifndef BL_NS
#error "compile with -DBL_NS=fast or -DBL_NS=exact"
#endif
#include "hydro_kernels.cuh"
#include "ale_kernels.cuh"
