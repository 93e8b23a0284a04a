// Intra lattice kernel instances for CUs 64 samples wide (heights 4..64).
#include "lattice_kernel.cuh"

namespace uc {

template <>
int lat_launch_w<6>(int lh, unsigned grid, int smem, cudaStream_t st, const LatParams &P)
{
    static bool attr[64][7];
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "intra_lattice: device index");
    void (*k)(LatParams) = nullptr;
    switch (lh) {
    case 2: k = k_intra_lattice<6, 2>; break;
    case 3: k = k_intra_lattice<6, 3>; break;
    case 4: k = k_intra_lattice<6, 4>; break;
    case 5: k = k_intra_lattice<6, 5>; break;
    case 6: k = k_intra_lattice<6, 6>; break;
    default: return set_status(UC_ERR_ARG, "intra_lattice: CU height");
    }
    // the launch's own size decides the occupancy; the attribute only has to admit every
    // layout (mode counts change it)
    if (!attr[dev][lh]) {
        UC_CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, LAT_SMEM_MAX));
        attr[dev][lh] = true;
    }
    if (smem > LAT_SMEM_MAX) return set_status(UC_ERR_ARG, "intra_lattice: shared memory layout");
    k<<<grid, LAT_THREADS, smem, st>>>(P);
    UC_CHECK(cudaGetLastError());
    return UC_OK;
}

}  // namespace uc
