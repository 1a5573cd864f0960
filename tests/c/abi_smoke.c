/* The C ABI from plain C (include/logo_gpu.h): create a context, one best
 * move, a descent, a tour length, an ILS run, the device start tours, the
 * neighbour-list search and the route transfer modes, destroy.  Reads an
 * instance from argv[1] (uint32 n, then n x (float x, float y), then n
 * uint32 route) and prints one line per result for the test to compare with
 * the oracle and the host builders:
 *   move <minchange> <i> <j>
 *   descend <moves> <final_length> <route...>
 *   length <length of the descended tour>
 *   ils <best_length> <moves> <accepted> <route...>
 *   nnstart <route...>      (logo_start_tour, LOGO_START_NN)
 *   mfstart <route...>      (logo_start_tour, LOGO_START_MF)
 *   nbrdescend <moves> <final_length> <route...>  (LOGO_SEARCH_NEIGHBOUR, 8)
 *   copydescend <moves> <final_length>            (LOGO_ROUTE_IO_COPY)
 * Exit status 0 on success, 1 on a usage or file error, 2 on a library error. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "logo_gpu.h"

static int fail(logo_ctx *ctx, const char *what, logo_status s) {
    fprintf(stderr, "%s: status %d: %s\n", what, (int)s, logo_last_error(ctx));
    return 2;
}

int main(int argc, char **argv) {
    if (argc < 2) return 1;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 1;
    uint32_t n = 0;
    if (fread(&n, 4, 1, f) != 1 || n < 3) return 1;
    logo_xy *xy = (logo_xy *)malloc(sizeof(logo_xy) * n);
    uint32_t *route = (uint32_t *)malloc(4u * n), *start = (uint32_t *)malloc(4u * n);
    if (!xy || !route || !start) return 1;
    if (fread(xy, sizeof(logo_xy), n, f) != n || fread(start, 4, n, f) != n) return 1;
    fclose(f);

    logo_ctx *ctx = NULL;
    logo_status s = logo_ctx_create(0, xy, n, &ctx);
    if (s != LOGO_OK) return fail(NULL, "logo_ctx_create", s);
    logo_move m;
    s = logo_best_move(ctx, start, &m);
    if (s != LOGO_OK) return fail(ctx, "logo_best_move", s);
    printf("move %d %u %u\n", m.minchange, m.i, m.j);

    logo_stats st;
    memcpy(route, start, 4u * n);
    s = logo_descend(ctx, route, 0, &st);
    if (s != LOGO_OK) return fail(ctx, "logo_descend", s);
    printf("descend %llu %llu", (unsigned long long)st.moves, (unsigned long long)st.final_length);
    for (uint32_t k = 0; k < n; ++k) printf(" %u", route[k]);
    printf("\n");

    uint64_t len = 0;
    s = logo_tour_length(ctx, route, &len);
    if (s != LOGO_OK) return fail(ctx, "logo_tour_length", s);
    printf("length %llu\n", (unsigned long long)len);

    memcpy(route, start, 4u * n);
    s = logo_ils(ctx, route, 10, 99, LOGO_KICK_DOUBLE_BRIDGE, &st);
    if (s != LOGO_OK) return fail(ctx, "logo_ils", s);
    printf("ils %llu %llu %llu", (unsigned long long)st.final_length,
           (unsigned long long)st.moves, (unsigned long long)st.accepted);
    for (uint32_t k = 0; k < n; ++k) printf(" %u", route[k]);
    printf("\n");

    s = logo_start_tour(ctx, LOGO_START_NN, route);
    if (s != LOGO_OK) return fail(ctx, "logo_start_tour", s);
    printf("nnstart");
    for (uint32_t k = 0; k < n; ++k) printf(" %u", route[k]);
    printf("\n");
    s = logo_start_tour(ctx, LOGO_START_MF, route);
    if (s != LOGO_OK) return fail(ctx, "logo_start_tour", s);
    printf("mfstart");
    for (uint32_t k = 0; k < n; ++k) printf(" %u", route[k]);
    printf("\n");

    s = logo_ctx_set_search(ctx, LOGO_SEARCH_NEIGHBOUR, 8);
    if (s != LOGO_OK) return fail(ctx, "logo_ctx_set_search", s);
    memcpy(route, start, 4u * n);
    s = logo_descend(ctx, route, 0, &st);
    if (s != LOGO_OK) return fail(ctx, "logo_descend (neighbour search)", s);
    printf("nbrdescend %llu %llu", (unsigned long long)st.moves,
           (unsigned long long)st.final_length);
    for (uint32_t k = 0; k < n; ++k) printf(" %u", route[k]);
    printf("\n");
    s = logo_ctx_set_search(ctx, LOGO_SEARCH_EXHAUSTIVE, 0);
    if (s != LOGO_OK) return fail(ctx, "logo_ctx_set_search", s);

    s = logo_ctx_set_route_io(ctx, LOGO_ROUTE_IO_COPY);
    if (s != LOGO_OK) return fail(ctx, "logo_ctx_set_route_io", s);
    memcpy(route, start, 4u * n);
    s = logo_descend(ctx, route, 0, &st);
    if (s != LOGO_OK) return fail(ctx, "logo_descend (copied route)", s);
    printf("copydescend %llu %llu\n", (unsigned long long)st.moves,
           (unsigned long long)st.final_length);

    s = logo_ctx_destroy(ctx);
    if (s != LOGO_OK) return fail(NULL, "logo_ctx_destroy", s);
    free(xy);
    free(route);
    free(start);
    return 0;
}
