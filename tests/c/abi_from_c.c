/* The C ABI used from plain C99: builds the reference's shipped cylinder case on the host
 * (mrlbm_create_host needs no GPU), prints its boundary counts and checks an error path.
 * Compiled and run by tests/test_abi.py. */
#include <stdio.h>
#include <string.h>

#include "mrlbm.h"

int main(void) {
    mrlbm_case_desc d;
    if (mrlbm_case_desc_default(&d, MRLBM_GEOM_CYLINDER) != MRLBM_OK) return 1;
    if (mrlbm_case_desc_finalize(&d) != MRLBM_OK) {
        fprintf(stderr, "%s\n", mrlbm_last_error(NULL));
        return 2;
    }
    mrlbm_handle *h = NULL;
    if (mrlbm_create_host(&d, &h) != MRLBM_OK) {
        fprintf(stderr, "%s\n", mrlbm_last_error(NULL));
        return 3;
    }
    mrlbm_info info;
    if (mrlbm_get_info(h, &info) != MRLBM_OK) return 4;
    /* a host-only handle refuses device work with a status, it does not exit */
    const int rc = mrlbm_step(h, 1);
    printf("%d %d %d %d %d %d %s\n", info.nx, info.ny, info.nz, info.nb[0], info.nb_fluid[0], rc,
           rc != MRLBM_OK && strlen(mrlbm_last_error(h)) > 0 ? "error-reported" : "no-error");
    mrlbm_destroy(h);

    /* the case of the INTEGRATION example: another grid and body, window derived */
    if (mrlbm_case_desc_default(&d, MRLBM_GEOM_CYLINDER) != MRLBM_OK) return 5;
    d.nx = 128; d.ny = 64; d.nz = 32; d.xc = 32; d.yc = 32; d.d_wall[0] = 16; d.re = 100; d.u_max = 0.05f;
    memset(d.scan_box, 0, sizeof(d.scan_box));
    if (mrlbm_case_desc_finalize(&d) != MRLBM_OK || mrlbm_create_host(&d, &h) != MRLBM_OK) {
        fprintf(stderr, "%s\n", mrlbm_last_error(NULL));
        return 6;
    }
    if (mrlbm_get_info(h, &info) != MRLBM_OK) return 7;
    printf("%d %d %d %d %d\n", d.scan_box[0], d.scan_box[1], d.scan_box[2], d.scan_box[3], info.nb[0]);
    mrlbm_destroy(h);
    return 0;
}
