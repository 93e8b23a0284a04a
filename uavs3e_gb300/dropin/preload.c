/*
 * preload.c -- runs an unchanged uavs3e encoder on libuavs3e_cuda's kernel-table entries.
 *
 * Built as libuavs3e_cuda_preload.so next to libuavs3e_cuda.so.  Loaded with LD_PRELOAD into a
 * program linked against the encoder (e.g. its uavs3enc application), it wraps uavs3e_create
 * (src/uavs3e.c:1266): the encoder fills its global kernel table uavs3e_funs_handle
 * (src/com_util.c:40) there from uavs3e_funs_init_c/_sse/_avx2 (src/uavs3e.c:1332-1339), and
 * right after that the wrapper calls uavs3e_cuda_install() on it, which points every hot-path
 * member at the GPU entries.  This is the line an integrator adds after uavs3e_create in their
 * own code; the preload does it without rebuilding the encoder.
 *
 * At exit it prints one line to stderr: the library's status (0 = every call succeeded) and the
 * number of kernels it launched.  With UAVS3E_CUDA_COSTLOG=1 in the environment it also records
 * every cost call (costlog.h) and prints the record's counts and hash at exit.
 *
 *   LD_PRELOAD=.../libuavs3e_cuda_preload.so uavs3enc ...
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../include/uavs3e_cuda_table.h"
#include "costlog.h"

static int g_installed;

static void report(void)
{
    if (!g_installed) return;
    fprintf(stderr, "uavs3e_cuda_preload: status %d (%s), %llu kernel launches\n", uavs3e_cuda_status(),
            uavs3e_cuda_status_string(), uavs3e_cuda_launch_count());
}

void *uavs3e_create(void *cfg, int *err)
{
    void *(*real)(void *, int *) = (void *(*)(void *, int *))dlsym(RTLD_NEXT, "uavs3e_create");
    if (!real) {
        fprintf(stderr, "uavs3e_cuda_preload: uavs3e_create not found in the program\n");
        exit(3);
    }
    void *h = real(cfg, err);
    if (!h) return h;
    void *table = dlsym(RTLD_DEFAULT, "uavs3e_funs_handle");
    if (!table) {
        fprintf(stderr, "uavs3e_cuda_preload: uavs3e_funs_handle not found in the program\n");
        exit(3);
    }
    int rc = uavs3e_cuda_install(table);
    if (rc) {
        /* no CPU fallback: an encoder that cannot run on the GPU entries stops here */
        fprintf(stderr, "uavs3e_cuda_preload: install failed (%d): %s\n", rc, uavs3e_cuda_status_string());
        exit(4);
    }
    if (getenv("UAVS3E_CUDA_COSTLOG") && getenv("UAVS3E_CUDA_COSTLOG")[0] == '1') costlog_install(table);
    if (!g_installed) atexit(report);
    g_installed = 1;
    fprintf(stderr, "uavs3e_cuda_preload: kernel table installed (GPU entries)\n");
    return h;
}
