/* A C caller of the C ABI (include/sphstokes.h), as a compiled host program would bind it:
 * the default spherical diapir parameters on a 15 x 13 x 11 grid, k reference PT
 * iterations in FP64 (sph_step replaces the loop body of SphericalStokes_diapir.jl:413-425),
 * then the pressure field (sph_get_field, the reference's layout) and the FP64 residual.
 * Prints "P <max|P|> <sum P> residual <err>" and returns 0, or prints the library's error
 * and returns 1.  Usage: c_caller [k]  (k = 10 by default). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "sphstokes.h"

static int check(int rc, const char* what) {
    if (rc != 0) fprintf(stderr, "%s: %s (%s)\n", what, sph_strerror(rc), sph_last_error());
    return rc != 0;
}

int main(int argc, char** argv) {
    const long long k = argc > 1 ? atoll(argv[1]) : 10;
    sph_params p;
    if (check(sph_params_default(&p, SPH_GEOM_SPHERICAL), "sph_params_default")) return 1;
    p.n1 = 15; p.n2 = 13; p.n3 = 11;
    p.precision = SPH_PREC_FP64;
    int64_t dims[3];
    if (check(sph_field_dims(&p, SPH_FIELD_P, dims), "sph_field_dims")) return 1;
    const int64_t count = dims[0] * dims[1] * dims[2];
    double* P = (double*)malloc(sizeof(double) * (size_t)count);
    void* ctx = NULL;
    if (!P || check(sph_create(&p, &ctx), "sph_create")) return 1;
    double out[7];
    int bad = check(sph_step(ctx, k), "sph_step") || check(sph_get_field(ctx, SPH_FIELD_P, P, count), "sph_get_field") ||
              check(sph_residual(ctx, out), "sph_residual");
    sph_destroy(ctx);
    if (bad) return 1;
    double mx = 0.0, sum = 0.0;
    for (int64_t i = 0; i < count; ++i) {
        mx = fmax(mx, fabs(P[i]));
        sum += P[i];
    }
    printf("P %.17g %.17g residual %.17g\n", mx, sum, out[6]);
    free(P);
    return 0;
}
