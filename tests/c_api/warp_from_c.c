/* A C caller of libidwarp_gb300.so (include/idwarp_gb300.h): a cube surface
 * and a shell of volume points, surface definition through idw_point_reduce,
 * a rigid translation warp (every volume node must move by the translation)
 * and the translation identity of the reverse product (sum dXs = sum dXv);
 * then the restart-file path: a second context loads the first one's
 * denominator estimate (a tampered copy is refused) and warps to the same
 * bits.  Exit status 0 on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "idwarp_gb300.h"

#define N 6     /* quads per cube edge */
#define LAYERS 5

static const double *g_u;
static int cmp_zyx(const void *a, const void *b) {
    const double *p = g_u + 3 * *(const int *)a, *q = g_u + 3 * *(const int *)b;
    for (int k = 2; k >= 0; --k) {
        if (p[k] < q[k]) return -1;
        if (p[k] > q[k]) return 1;
    }
    return 0;
}

static int check(void *ctx, int rc, const char *what) {
    if (rc != IDW_OK) {
        char msg[512];
        idw_last_error(ctx, msg, sizeof msg);
        fprintf(stderr, "%s failed (%d): %s\n", what, rc, msg);
        exit(1);
    }
    return rc;
}

int main(void) {
    /* six cube faces, (N+1)^2 points each (edges duplicated), N^2 quads each */
    const int ppf = (N + 1) * (N + 1), npts = 6 * ppf, nfaces = 6 * N * N;
    double *pts = malloc(sizeof(double) * 3 * npts);
    int32_t *conn = malloc(sizeof(int32_t) * 4 * nfaces), *fs = malloc(sizeof(int32_t) * nfaces);
    int f = 0;
    for (int face = 0; face < 6; ++face) {
        const int ax = face / 2, s = (face % 2) ? 1 : -1, u = (ax + 1) % 3, v = (ax + 2) % 3;
        for (int i = 0; i <= N; ++i)
            for (int j = 0; j <= N; ++j) {
                double *p = pts + 3 * (face * ppf + i * (N + 1) + j);
                p[ax] = s;
                p[u] = -1.0 + 2.0 * i / N;
                p[v] = -1.0 + 2.0 * j / N;
            }
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const int a = face * ppf + i * (N + 1) + j;
                int32_t *q = conn + 4 * f;
                if (s > 0) { q[0] = a; q[1] = a + N + 1; q[2] = a + N + 2; q[3] = a + 1; }
                else { q[0] = a; q[1] = a + 1; q[2] = a + N + 2; q[3] = a + N + 1; }
                fs[f++] = 4;
            }
    }
    /* volume: the surface points scaled outwards in LAYERS shells */
    const int nvol = LAYERS * npts;
    double *xv0 = malloc(sizeof(double) * 3 * nvol);
    for (int l = 0; l < LAYERS; ++l)
        for (int k = 0; k < 3 * npts; ++k) xv0[3 * l * npts + k] = pts[k] * (1.0 + 0.5 * (l + 1));

    idw_options o;
    idw_default_options(&o);
    o.precision = IDW_PREC_MIXED;
    void *ctx = NULL;
    if (idw_create(&o, &ctx) != IDW_OK) { fprintf(stderr, "idw_create failed\n"); return 1; }
    check(ctx, idw_create_common_grid(ctx, xv0, nvol, IDW_HOST), "create_common_grid");
    check(ctx, idw_set_symmetry_planes(ctx, NULL, NULL, 0), "set_symmetry_planes");

    /* unique points, sorted by z, then y, then x; link is 1-based */
    double *uniq = malloc(sizeof(double) * 3 * npts);
    int32_t *link = malloc(sizeof(int32_t) * npts), nu = 0;
    check(ctx, idw_point_reduce(pts, npts, 1e-12, uniq, link, &nu), "point_reduce");
    int *ord = malloc(sizeof(int) * nu), *inv = malloc(sizeof(int) * nu);
    for (int i = 0; i < nu; ++i) ord[i] = i;
    g_u = uniq;
    qsort(ord, nu, sizeof(int), cmp_zyx);
    double *sorted = malloc(sizeof(double) * 3 * nu);
    for (int i = 0; i < nu; ++i) {
        inv[ord[i]] = i;
        for (int k = 0; k < 3; ++k) sorted[3 * i + k] = uniq[3 * ord[i] + k];
    }
    for (int i = 0; i < npts; ++i) link[i] = inv[link[i] - 1] + 1;
    check(ctx, idw_initialize_warping(ctx, pts, npts, sorted, nu, link, fs, nfaces, conn, 4 * nfaces),
          "initialize_warping");

    /* rigid translation of the surface */
    const double t[3] = {0.25, -0.125, 0.5};
    double *xs = malloc(sizeof(double) * 3 * npts);
    for (int i = 0; i < npts; ++i)
        for (int k = 0; k < 3; ++k) xs[3 * i + k] = pts[3 * i + k] + t[k];
    check(ctx, idw_set_surface_coordinates(ctx, xs, 3 * npts, IDW_HOST), "set_surface_coordinates");
    check(ctx, idw_warp_mesh(ctx), "warp_mesh");
    double *xv = malloc(sizeof(double) * 3 * nvol);
    check(ctx, idw_get_volume_coordinates(ctx, xv, 3 * nvol, IDW_HOST), "get_volume_coordinates");
    double err = 0.0;
    for (int i = 0; i < nvol; ++i)
        for (int k = 0; k < 3; ++k) err = fmax(err, fabs(xv[3 * i + k] - xv0[3 * i + k] - t[k]));

    /* reverse product of dXv = 1: a uniform translation of the surface moves every node */
    double *dxv = malloc(sizeof(double) * 3 * nvol), *dxs = malloc(sizeof(double) * 3 * npts);
    for (int k = 0; k < 3 * nvol; ++k) dxv[k] = 1.0;
    check(ctx, idw_warp_deriv(ctx, dxv, 3 * nvol, IDW_HOST), "warp_deriv");
    check(ctx, idw_get_dxs(ctx, dxs, 3 * npts, IDW_HOST), "get_dxs");
    double sum = 0.0;
    for (int k = 0; k < 3 * npts; ++k) sum += dxs[k];
    idw_stats st;
    check(ctx, idw_get_stats(ctx, &st), "get_stats");

    /* restart: the estimate and the dryRun costs of this context ... */
    double *den0 = malloc(sizeof(double) * nvol), *costs = malloc(sizeof(double) * nvol);
    check(ctx, idw_get_denominator0(ctx, den0, nvol, IDW_HOST), "get_denominator0");
    check(ctx, idw_dry_run_costs(ctx, costs, nvol, IDW_HOST), "dry_run_costs");
    idw_destroy(ctx);
    for (int i = 0; i < nvol; ++i)
        if (!(costs[i] > 0.0)) return 6;
    /* ... loaded by a second one in place of computing it */
    void *ctx2 = NULL;
    if (idw_create(&o, &ctx2) != IDW_OK) { fprintf(stderr, "idw_create failed\n"); return 1; }
    check(ctx2, idw_create_common_grid(ctx2, xv0, nvol, IDW_HOST), "create_common_grid (2)");
    check(ctx2, idw_set_symmetry_planes(ctx2, NULL, NULL, 0), "set_symmetry_planes (2)");
    check(ctx2, idw_initialize_warping(ctx2, pts, npts, sorted, nu, link, fs, nfaces, conn, 4 * nfaces),
          "initialize_warping (2)");
    den0[0] *= 2.0; /* node 0 is checked: an estimate above the truth is refused */
    if (idw_set_denominator0(ctx2, den0, nvol, 100, IDW_HOST) != IDW_ERR_RESTART) return 4;
    den0[0] *= 0.5;
    check(ctx2, idw_set_denominator0(ctx2, den0, nvol, 100, IDW_HOST), "set_denominator0");
    check(ctx2, idw_set_surface_coordinates(ctx2, xs, 3 * npts, IDW_HOST), "set_surface_coordinates (2)");
    check(ctx2, idw_warp_mesh(ctx2), "warp_mesh (2)");
    double *xv2 = malloc(sizeof(double) * 3 * nvol);
    check(ctx2, idw_get_volume_coordinates(ctx2, xv2, 3 * nvol, IDW_HOST), "get_volume_coordinates (2)");
    idw_destroy(ctx2);
    if (memcmp(xv, xv2, sizeof(double) * 3 * nvol) != 0) return 5;
    printf("nvol %d nunique %d translation error %.3e sum(dXs) %.12g expected %d leafPairs %lld\n", nvol, nu, err,
           sum, 3 * nvol, (long long)st.leafPairs);
    if (!(err < 1e-12)) return 2;
    if (!(fabs(sum - 3.0 * nvol) < 1e-6 * 3.0 * nvol)) return 3;
    return 0;
}
