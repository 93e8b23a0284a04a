// Quantisation step table shared by the lattice and RDOQ kernels.
#pragma once
#include "common.cuh"

namespace uc {

// enc_tbl_quant_scale (src/quant.c:55-66): quantisation scale per step index 0..79
__device__ __constant__ static const u16 kQScale[80] = {
    16302, 15024, 13777, 12634, 11626, 10624, 9742, 8958, 8192, 7512, 6889, 6305, 5793, 5303, 4878, 4467,
    4091, 3756, 3444, 3161, 2894, 2654, 2435, 2235, 2048, 1878, 1722, 1579, 1449, 1329, 1218, 1117,
    1024, 939, 861, 790, 724, 664, 609, 558, 512, 470, 430, 395, 362, 332, 304, 279,
    256, 235, 215, 197, 181, 166, 152, 140, 128, 116, 108, 99, 91, 83, 76, 69,
    64, 59, 54, 49, 45, 41, 38, 35, 32, 30, 27, 25, 23, 21, 19, 18,
};

}  // namespace uc
