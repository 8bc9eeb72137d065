/* A plain C99 caller of the library, the way a Swift, Go or C host binds it:
 * the header compiles as C, the library links, and the status conventions
 * hold. Without a CUDA device stro_ctx_create must return STRO_ERR_NO_DEVICE
 * with a message; with one, a small periodic Taylor-Green box is stepped and
 * its digest printed. Exit status 0 on the expected behaviour. */
#include <stdio.h>
#include <string.h>

#include "strouhal_c.h"

int main(void) {
    stro_ctx* ctx = NULL;
    int rc = stro_ctx_create(0, &ctx);
    if (rc == STRO_ERR_NO_DEVICE) {
        const char* msg = stro_last_error();
        if (ctx != NULL || msg == NULL || msg[0] == '\0') return 2;
        printf("no-device %s\n", msg);
        return 0;
    }
    if (rc != STRO_OK) return 3;
    stro_sim_desc d;
    memset(&d, 0, sizeof d);
    d.precision = STRO_FP32;
    d.nx = 32;
    d.ny = 16;
    d.nz = 8;
    d.omega = 1.8f;
    d.omega_minus = 1.8f;
    stro_sim* sim = NULL;
    char hex[65];
    double mass = 0.0;
    rc = stro_sim_create(ctx, &d, NULL, &sim);
    if (rc == STRO_OK) rc = stro_sim_init_field(sim, 2, 0.05f);
    if (rc == STRO_OK) rc = stro_sim_run(sim, 10);
    if (rc == STRO_OK) rc = stro_sim_digest(sim, hex);
    if (rc == STRO_OK) rc = stro_sim_mass(sim, &mass);
    if (rc == STRO_OK) printf("digest %s mass %.17g\n", hex, mass);
    else fprintf(stderr, "error %d: %s\n", rc, stro_last_error());
    if (sim) stro_sim_destroy(sim);
    stro_ctx_destroy(ctx);
    return rc == STRO_OK ? 0 : 4;
}
