/*
 * costlog.h -- a record of every cost call an encoder makes through its kernel table.
 *
 * costlog_install() wraps the table's current cost members -- cost_sad, cost_sad_x3, cost_sad_x4,
 * cost_ssd (each [log2(w) - 2]) and cost_satd[log2(w) - 2][log2(h) - 2] (funs_handle_t,
 * inc/com_util.h:316-322) -- with functions that call the wrapped member and fold
 * (member, width index, height, result) into a running 64-bit FNV-1a hash, and count the calls
 * per member family.  At exit it prints one line to stderr:
 *
 *   costlog: sad <n> sad_x3 <n> sad_x4 <n> ssd <n> satd <n> hash <16 hex digits>
 *
 * Two encodes of the same input whose cost members return the same value for every call, in the
 * same order, print the same line; the first differing call changes the hash.  The record is
 * ordered, so it is meant for single-threaded encodes (--wpp_threads 1 --frm_threads 1).
 * Include it in one translation unit; everything here is static.
 */
#ifndef UAVS3E_COSTLOG_H
#define UAVS3E_COSTLOG_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../include/uavs3e_cuda_table.h"

typedef uint32_t (*costlog_sad_t)(uint8_t *, int, uint8_t *, int, int);
typedef void (*costlog_sad3_t)(uint8_t *, int, uint8_t *, uint8_t *, uint8_t *, int, uint32_t *, int);
typedef void (*costlog_sad4_t)(uint8_t *, int, uint8_t *, uint8_t *, uint8_t *, uint8_t *, int, uint32_t *, int);
typedef uint64_t (*costlog_ssd_t)(uint8_t *, int, uint8_t *, int, int);
typedef uint32_t (*costlog_satd_t)(uint8_t *, int, uint8_t *, int);

static uint64_t costlog_h = 1469598103934665603ull;
static unsigned long long costlog_n[5];
static costlog_sad_t costlog_sad[6];
static costlog_sad3_t costlog_sad3[6];
static costlog_sad4_t costlog_sad4[6];
static costlog_ssd_t costlog_ssd[6];
static costlog_satd_t costlog_satd[3][3];

static void costlog_mix(uint64_t v)
{
    for (int i = 0; i < 8; i++) {
        costlog_h ^= (v >> (8 * i)) & 0xFF;
        costlog_h *= 1099511628211ull;
    }
}

static void costlog_rec(int fam, int a, int b, uint64_t r)
{
    costlog_mix(((uint64_t)fam << 48) | ((uint64_t)(a & 0xFF) << 40) | ((uint64_t)(b & 0xFFFF) << 16));
    costlog_mix(r);
    costlog_n[fam]++;
}

#define COSTLOG_W(M) M(0) M(1) M(2) M(3) M(4) M(5)
#define COSTLOG_SAD(i)                                                                          \
    static uint32_t costlog_sad_##i(uint8_t *o, int io, uint8_t *p, int ip, int h)              \
    {                                                                                           \
        const uint32_t r = costlog_sad[i](o, io, p, ip, h);                                     \
        costlog_rec(0, i, h, r);                                                                \
        return r;                                                                               \
    }
#define COSTLOG_SAD3(i)                                                                         \
    static void costlog_sad3_##i(uint8_t *o, int io, uint8_t *p0, uint8_t *p1, uint8_t *p2, int ip, \
                                 uint32_t s[3], int h)                                          \
    {                                                                                           \
        costlog_sad3[i](o, io, p0, p1, p2, ip, s, h);                                           \
        for (int k = 0; k < 3; k++) costlog_rec(1, i, h, s[k]);                                 \
    }
#define COSTLOG_SAD4(i)                                                                         \
    static void costlog_sad4_##i(uint8_t *o, int io, uint8_t *p0, uint8_t *p1, uint8_t *p2, uint8_t *p3, \
                                 int ip, uint32_t s[4], int h)                                  \
    {                                                                                           \
        costlog_sad4[i](o, io, p0, p1, p2, p3, ip, s, h);                                       \
        for (int k = 0; k < 4; k++) costlog_rec(2, i, h, s[k]);                                 \
    }
#define COSTLOG_SSD(i)                                                                          \
    static uint64_t costlog_ssd_##i(uint8_t *o, int io, uint8_t *p, int ip, int h)              \
    {                                                                                           \
        const uint64_t r = costlog_ssd[i](o, io, p, ip, h);                                     \
        costlog_rec(3, i, h, r);                                                                \
        return r;                                                                               \
    }
COSTLOG_W(COSTLOG_SAD) COSTLOG_W(COSTLOG_SAD3) COSTLOG_W(COSTLOG_SAD4) COSTLOG_W(COSTLOG_SSD)
#define COSTLOG_SATD(a, b)                                                                      \
    static uint32_t costlog_satd_##a##b(uint8_t *o, int io, uint8_t *p, int ip)                 \
    {                                                                                           \
        const uint32_t r = costlog_satd[a][b](o, io, p, ip);                                    \
        costlog_rec(4, a, b, r);                                                                \
        return r;                                                                               \
    }
COSTLOG_SATD(0, 0) COSTLOG_SATD(0, 1) COSTLOG_SATD(0, 2) COSTLOG_SATD(1, 0) COSTLOG_SATD(1, 1)
COSTLOG_SATD(1, 2) COSTLOG_SATD(2, 0) COSTLOG_SATD(2, 1) COSTLOG_SATD(2, 2)

static void costlog_report(void)
{
    fprintf(stderr, "costlog: sad %llu sad_x3 %llu sad_x4 %llu ssd %llu satd %llu hash %016llx\n", costlog_n[0],
            costlog_n[1], costlog_n[2], costlog_n[3], costlog_n[4], (unsigned long long)costlog_h);
}

/* wraps the table's current cost members; a table whose members are already wrapped is left as
 * it is (the record and the counts are kept for the whole process) */
static void costlog_install(uavs3e_cuda_funs_t *t)
{
    static int registered;
    if (t->cost_sad[0] == costlog_sad_0) return;
    if (!registered) atexit(costlog_report);
    registered = 1;
#define COSTLOG_SET(i)                                                                          \
    costlog_sad[i] = t->cost_sad[i]; if (t->cost_sad[i]) t->cost_sad[i] = costlog_sad_##i;        \
    costlog_sad3[i] = t->cost_sad_x3[i]; if (t->cost_sad_x3[i]) t->cost_sad_x3[i] = costlog_sad3_##i; \
    costlog_sad4[i] = t->cost_sad_x4[i]; if (t->cost_sad_x4[i]) t->cost_sad_x4[i] = costlog_sad4_##i; \
    costlog_ssd[i] = t->cost_ssd[i]; if (t->cost_ssd[i]) t->cost_ssd[i] = costlog_ssd_##i;
    COSTLOG_W(COSTLOG_SET)
#undef COSTLOG_SET
#define COSTLOG_SETS(a, b)                                                                      \
    costlog_satd[a][b] = t->cost_satd[a][b]; if (t->cost_satd[a][b]) t->cost_satd[a][b] = costlog_satd_##a##b;
    COSTLOG_SETS(0, 0) COSTLOG_SETS(0, 1) COSTLOG_SETS(0, 2) COSTLOG_SETS(1, 0) COSTLOG_SETS(1, 1)
    COSTLOG_SETS(1, 2) COSTLOG_SETS(2, 0) COSTLOG_SETS(2, 1) COSTLOG_SETS(2, 2)
#undef COSTLOG_SETS
}

#endif
