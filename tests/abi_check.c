/*
 * abi_check.c -- test harness (not part of the library).
 *
 * A plain C99 consumer of librchem_gpu.so, as a bindgen- or FFI-generated
 * binding sees it: it includes the public headers in C mode, links the shared
 * library and calls the entry points that need no GPU (the ABI version, the
 * packed-index helper of libpyquante2's cints.h, argument validation with
 * status codes and rchem_last_error).  Exit status 0 on success; the failing
 * check is printed otherwise.
 */
#include <stdio.h>
#include <string.h>

#include "rchem_cints.h"
#include "rchem_gpu.h"

static int failures = 0;

#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            fprintf(stderr, "abi_check: %s:%d: %s\n", __FILE__, __LINE__, #cond); \
            ++failures;                                              \
        }                                                            \
    } while (0)

/* cints.c:375-387: the position of (ij|kl) in the 8-fold packed tensor */
static long long pack8(long long i, long long j, long long k, long long l) {
    long long t, ij, kl;
    if (i < j) { t = i; i = j; j = t; }
    if (k < l) { t = k; k = l; l = t; }
    ij = i * (i + 1) / 2 + j;
    kl = k * (k + 1) / 2 + l;
    if (ij < kl) { t = ij; ij = kl; kl = t; }
    return ij * (ij + 1) / 2 + kl;
}

int main(void) {
    int i, j, k, l, rc;
    rchem_basis h = NULL;
    const int Z[1] = {8};
    const double R[3] = {0.0, 0.0, 0.0};
    const int atom[1] = {0}, lval[1] = {3}, nprim[1] = {1};
    const double e[1] = {1.0}, c[1] = {1.0};

    CHECK(rchem_abi_version() == 1);
    for (i = 0; i < 6; ++i)
        for (j = 0; j < 6; ++j)
            for (k = 0; k < 6; ++k)
                for (l = 0; l < 6; ++l) {
                    CHECK(ijkl2intindex(i, j, k, l) == (int)pack8(i, j, k, l));
                    CHECK(ijkl2intindex(i, j, k, l) == ijkl2intindex(k, l, j, i));
                }

    /* an f shell: refused with a status code and a message, no handle */
    rc = rchem_basis_create(&h, 1, Z, R, 1, atom, lval, nprim, e, c);
    CHECK(rc == RCHEM_ERR_UNSUPPORTED);
    CHECK(h == NULL);
    CHECK(rchem_last_error() != NULL && strstr(rchem_last_error(), "l=3") != NULL);
    /* null arguments */
    CHECK(rchem_jk_direct(NULL, NULL, NULL, NULL, NULL) == RCHEM_ERR_INVALID);
    CHECK(rchem_basis_nbf(NULL) == -1);
    CHECK(rchem_jk_inmem(0, NULL, NULL, NULL, NULL, RCHEM_HOST) == RCHEM_ERR_INVALID);

    if (failures) {
        fprintf(stderr, "abi_check: %d failure(s)\n", failures);
        return 1;
    }
    printf("abi_check: ok\n");
    return 0;
}
