// Definitions of the opaque C-ABI handle types shared by the translation units of the library.
#pragma once
#include <cuda_runtime.h>

#include "imps_internal.h"

struct imps_layout {
  imps::Layout L;
  // device copies of the block table (BlockDiagMat traces), uploaded on first use
  int64_t* d_boff = nullptr;
  int32_t* d_bdim = nullptr;
  ~imps_layout() {
    if (d_boff) cudaFree(d_boff);
    if (d_bdim) cudaFree(d_bdim);
  }
};
