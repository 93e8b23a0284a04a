// Host-built transform and scan tables, uploaded once per device.
//
// The integer DCT2/DCT8/DST7 matrices are the encoder's (com_dct_coef_create,
// src/com_tables.c:222-278: sqrt(N)*32 times the orthonormal basis, rounded half away from
// zero), frozen as constant data in dct_matrices.inc (gen_dct_matrices.py) rather than
// recomputed with the host's cos() at start-up.  The DCT2 partial butterflies of the encoder
// (src/transform.c:57-251, src/com_itdq.c:47-262) only read the first N/2^(l+1) entries of each
// row and rebuild the rest by even/odd symmetry; fold_dct2() builds the matrix those
// butterflies effectively apply, so the kernels can use plain matrix products with results
// identical to the butterflies.  The 4-point DCT8/DST7 use the fast forms of
// src/transform.c:416-432, 545-562 (inverse src/com_itdq.c:428-452, 543-566).
#include "common.cuh"
#include "tables.h"

#include <string.h>
#include <vector>

namespace uc {

#include "dct_matrices.inc"

// even/odd decomposition run on unit vectors: row k uses the difference vector of level
// ctz(k)+1, rows 0 and N/2 the final two-entry sum vector
static void fold_dct2(int L, const s8 *tm, s8 *F)
{
    int N = 1 << L;
    for (int n = 0; n < N; n++) {
        int S[7][64], D[7][64];
        for (int i = 0; i < N; i++) S[0][i] = i == n;
        for (int l = 1; l < L; l++) {
            int len = N >> (l - 1);
            for (int i = 0; i < len / 2; i++) {
                S[l][i] = S[l - 1][i] + S[l - 1][len - 1 - i];
                D[l][i] = S[l - 1][i] - S[l - 1][len - 1 - i];
            }
        }
        for (int k = 0; k < N; k++) {
            const int *V;
            int len;
            if (k == 0 || k == N / 2) { V = S[L - 1]; len = 2; }
            else { int j = __builtin_ctz(k); V = D[j + 1]; len = N >> (j + 1); }
            int acc = 0;
            for (int i = 0; i < len; i++) acc += tm[k * N + i] * V[i];
            F[k * N + n] = (s8)acc;   // each entry is +-one table entry
        }
    }
}

static void eff_dct87(int L, const s8 *T, s16 *M8, s16 *M7)
{
    int N = 1 << L;
    const s8 *d8 = T + 1 * N * N, *d7 = T + 2 * N * N;
    if (N == 4) {
        int b = d8[1], c = d8[2], d = d8[3];
        int r8[16] = { c + d, b, c, d, b, 0, -b, -b, c, -b, -d, c + d, d, -b, c + d, -c };
        int a = d7[0], b7 = d7[1], c7 = d7[2];
        int r7[16] = { a, b7, c7, a + b7, c7, c7, 0, -c7, a + b7, -a, -c7, b7, b7, -(a + b7), c7, -a };
        for (int i = 0; i < 16; i++) { M8[i] = (s16)r8[i]; M7[i] = (s16)r7[i]; }
    } else {
        for (int i = 0; i < N * N; i++) { M8[i] = d8[i]; M7[i] = d7[i]; }
    }
}

// zig-zag scan (init_scan, src/com_util.c:1220-1252) and its inverse (raster -> scan index)
static void gen_scan(int lx, int ly, u16 *scan, u16 *pos)
{
    int sx = 1 << lx, sy = 1 << ly, p = 0;
    scan[p++] = 0;
    for (int l = 1; l < sx + sy - 1; l++) {
        if (l & 1) {
            int x = l < sx - 1 ? l : sx - 1, y = l - (sx - 1) > 0 ? l - (sx - 1) : 0;
            for (; x >= 0 && y < sy; x--, y++) scan[p++] = (u16)(y * sx + x);
        } else {
            int y = l < sy - 1 ? l : sy - 1, x = l - (sy - 1) > 0 ? l - (sy - 1) : 0;
            for (; y >= 0 && x < sx; x++, y--) scan[p++] = (u16)(y * sx + x);
        }
    }
    for (int i = 0; i < sx * sy; i++) pos[scan[i]] = (u16)i;
}

static DevTables g_tab[64];
static bool g_tab_ok[64];
static HostTables g_host;
static bool g_host_ok = false;

const HostTables &host_tables()
{
    if (!g_host_ok) {
        for (int L = 1; L <= 6; L++) memcpy(g_host.dct[L], kDctMat[L], (size_t)3 << (2 * L));
        for (int L = 2; L <= 6; L++) {
            fold_dct2(L, g_host.dct[L], g_host.fold[L]);
            eff_dct87(L, g_host.dct[L], g_host.d87[0][L], g_host.d87[1][L]);
        }
        for (int ly = 1; ly <= 6; ly++)
            for (int lx = 1; lx <= 6; lx++) gen_scan(lx, ly, g_host.scan[lx][ly], g_host.scanpos[lx][ly]);
        g_host_ok = true;
    }
    return g_host;
}

const DevTables *device_tables(int dev)
{
    if (dev < 0 || dev >= 64) return nullptr;
    if (g_tab_ok[dev]) return &g_tab[dev];
    const HostTables &h = host_tables();
    void *buf = nullptr;
    if (cudaMalloc(&buf, sizeof(HostTables)) != cudaSuccess) return nullptr;
    if (cudaMemcpy(buf, &h, sizeof(HostTables), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    const HostTables *d = (const HostTables *)buf;
    DevTables &t = g_tab[dev];
    for (int L = 0; L <= 6; L++) {
        t.fold[L] = &d->fold[L][0];
        t.d87[0][L] = &d->d87[0][L][0];
        t.d87[1][L] = &d->d87[1][L][0];
        for (int M = 0; M <= 6; M++) { t.scanpos[L][M] = &d->scanpos[L][M][0]; t.scan[L][M] = &d->scan[L][M][0]; }
    }
    g_tab_ok[dev] = true;
    return &t;
}

}  // namespace uc
