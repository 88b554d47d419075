// main.cpp -- acum_gb300, the host program that replaces the reference driver
// (main.cu): reads the deck from the working directory (or the directory given), runs the
// broadband and tonal paths through the C ABI and writes pT.out, pL.out, pA.out and, with
// BB_noise = 1, bb_oaspl.out and bb_spl.dat.
//
//   acum_gb300 [deck_dir] [--fp64] [--device N]
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "acum.h"

int main(int argc, char** argv)
{
    const char* dir = ".";
    int precision = ACUM_MIXED, device = 0;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--fp64")) precision = ACUM_PLAIN_FP64;
        else if (!strcmp(argv[i], "--device") && i + 1 < argc) device = atoi(argv[++i]);
        else dir = argv[i];
    }
    acum_ctx* ctx = NULL;
    int rc = acum_create(&ctx, device);
    if (rc) {
        fprintf(stderr, "acum_gb300: %s\n", acum_last_global_error());
        return 1;
    }
    rc = acum_load_deck(ctx, dir);
    if (rc) {
        fprintf(stderr, "acum_gb300: %s\n", acum_last_error(ctx));
        return 1;
    }
    long long sz[6];
    acum_get_sizes(ctx, sz);
    printf("*** deck: %lld surfaces, %lld steps, %lld observers, %lld elements, %lld broadband sections\n", sz[0],
           sz[1], sz[2], sz[3], sz[4]);
    if (sz[5]) {
        double* spl = (double*)malloc(sizeof(double) * sz[2] * 42 * 7);
        double* oas = (double*)malloc(sizeof(double) * sz[2]);
        rc = acum_bpm(ctx, 0, spl, oas);
        free(spl);
        free(oas);
        if (rc) {
            fprintf(stderr, "acum_gb300: broadband: %s\n", acum_last_error(ctx));
            return 1;
        }
        double ms;
        if (acum_last_timing(ctx, 3, &ms, NULL) == ACUM_OK) printf("*** broadband kernels: %.3f ms\n", ms);
    }
    rc = acum_tonal(ctx, precision, NULL, NULL, NULL);
    if (rc) {
        fprintf(stderr, "acum_gb300: tonal: %s\n", acum_last_error(ctx));
        return 1;
    }
    double ms;
    if (acum_last_timing(ctx, 0, &ms, NULL) == ACUM_OK) printf("*** tonal kernel: %.3f ms\n", ms);
    uint32_t ew = 0;
    acum_device_error_word(ctx, &ew, 0);
    if (ew) printf("*** device error word: 0x%x\n", ew);
    rc = acum_write_outputs(ctx, dir);
    if (rc) {
        fprintf(stderr, "acum_gb300: %s\n", acum_last_error(ctx));
        return 1;
    }
    acum_destroy(ctx);
    printf("    DONE.....!\n");
    return 0;
}
