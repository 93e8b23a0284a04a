// Transform matrices and scan tables shared by the intra/transform kernels.
#pragma once
#include "common.cuh"

namespace uc {

// host copy (also the layout of the device copy)
struct HostTables {
    s8  dct[7][3 * 64 * 64];       // [log2N][type DCT2/DCT8/DST7][k][n]
    s8  fold[7][64 * 64];          // effective DCT2 matrix of the partial butterflies [k][n]
    s16 d87[2][7][64 * 64];        // effective DCT8 (0) / DST7 (1) matrices [k][n]
    u16 scan[7][7][64 * 64];       // [log2w][log2h] zig-zag scan: scan index -> raster
    u16 scanpos[7][7][64 * 64];    // [log2w][log2h] raster -> scan index
};

// device pointers into the uploaded copy
struct DevTables {
    const s8 *fold[7];
    const s16 *d87[2][7];
    const u16 *scan[7][7];
    const u16 *scanpos[7][7];
};

const HostTables &host_tables();
const DevTables *device_tables(int dev);   // uploads on first use; nullptr on failure

}  // namespace uc
