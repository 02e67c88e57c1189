/* plk_replay: a plain C caller of the engine's C ABI (include/plk.h), linked
 * against libplk.so and nothing else -- the calls treeator makes through
 * simpleML (src/treeator.cpp:715-724 set-up, :916 calculate_log_likelihood,
 * :973 draw_normalized_likelihood_on_nodes), made from C.
 *
 *   plk_replay <input> <output>
 *
 * input (little-endian): int32 n_tips, n_sites, n_states, n_nodes, n_cats,
 * root_quirk, reversible, p_mode; then uint32 masks[n_tips * n_sites],
 * int32 left[n_nodes], int32 right[n_nodes], double branch_length[n_nodes],
 * double Q[n_states^2], double root_weights[n_states], double
 * cat_rates[n_cats], double cat_weights[n_cats].
 * output: double lnL (FP64 plain form), double lnL (FP32 fast form), int32
 * n_internal, double node_states[n_internal * n_sites * n_states] (the
 * normalised conditional vectors, FP64), double site_lnl[n_sites] (FP64).
 * Exit status 0 on success; a failed call prints plk_last_error and exits 1. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "plk.h"

static int read_all(FILE* f, void* p, size_t size, size_t n) { return fread(p, size, n, f) == n; }

static void* alloc_or_die(size_t bytes) {
    void* p = malloc(bytes ? bytes : 1);
    if (!p) {
        fprintf(stderr, "plk_replay: out of host memory\n");
        exit(1);
    }
    return p;
}

#define CHECK(call)                                                                                   \
    do {                                                                                              \
        plk_status _s = (call);                                                                       \
        if (_s != PLK_OK) {                                                                           \
            fprintf(stderr, "plk_replay: %s failed: %s (%s)\n", #call, plk_status_string(_s),         \
                    plk_last_error(h));                                                               \
            return 1;                                                                                 \
        }                                                                                             \
    } while (0)

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: plk_replay <input> <output>\n");
        return 2;
    }
    FILE* in = fopen(argv[1], "rb");
    if (!in) {
        perror("plk_replay: input");
        return 1;
    }
    int32_t hd[8];
    if (!read_all(in, hd, sizeof(int32_t), 8)) {
        fprintf(stderr, "plk_replay: short header\n");
        return 1;
    }
    const int n_tips = hd[0], n_sites = hd[1], S = hd[2], n_nodes = hd[3], C = hd[4];
    const int root_quirk = hd[5], reversible = hd[6], p_mode = hd[7];
    if (n_tips < 1 || n_sites < 1 || S < 1 || S > 24 || n_nodes < n_tips || C < 1) {
        fprintf(stderr, "plk_replay: bad header\n");
        return 1;
    }
    uint32_t* masks = alloc_or_die(sizeof(uint32_t) * (size_t)n_tips * n_sites);
    int32_t* left = alloc_or_die(sizeof(int32_t) * n_nodes);
    int32_t* right = alloc_or_die(sizeof(int32_t) * n_nodes);
    double* bl = alloc_or_die(sizeof(double) * n_nodes);
    double* Q = alloc_or_die(sizeof(double) * S * S);
    double* rw = alloc_or_die(sizeof(double) * S);
    double* cr = alloc_or_die(sizeof(double) * C);
    double* cw = alloc_or_die(sizeof(double) * C);
    if (!read_all(in, masks, sizeof(uint32_t), (size_t)n_tips * n_sites) ||
        !read_all(in, left, sizeof(int32_t), n_nodes) || !read_all(in, right, sizeof(int32_t), n_nodes) ||
        !read_all(in, bl, sizeof(double), n_nodes) || !read_all(in, Q, sizeof(double), (size_t)S * S) ||
        !read_all(in, rw, sizeof(double), S) || !read_all(in, cr, sizeof(double), C) ||
        !read_all(in, cw, sizeof(double), C)) {
        fprintf(stderr, "plk_replay: short input\n");
        return 1;
    }
    fclose(in);

    plk_handle* h = NULL;
    CHECK(plk_create(&h, 0));
    CHECK(plk_set_alignment(h, n_tips, n_sites, S, masks));
    CHECK(plk_set_tree(h, n_nodes, left, right, bl));
    CHECK(plk_set_rate_model(h, root_quirk, 0, NULL, NULL, NULL, 0, NULL));
    CHECK(plk_set_model(h, S, Q, rw, reversible, C, cr, cw, p_mode));
    double lnl64 = 0.0, lnl32 = 0.0;
    CHECK(plk_loglik(h, PLK_FP32S, &lnl32));
    CHECK(plk_loglik(h, PLK_FP64, &lnl64));
    double* sites = alloc_or_die(sizeof(double) * n_sites);
    CHECK(plk_site_loglik(h, sites));
    const int32_t n_int = plk_n_internal(h);
    const size_t n_out = (size_t)n_int * n_sites * S;
    double* nodes = alloc_or_die(sizeof(double) * n_out);
    CHECK(plk_node_states(h, PLK_NODES_COND, PLK_FP64, nodes));
    plk_destroy(h);

    FILE* out = fopen(argv[2], "wb");
    if (!out) {
        perror("plk_replay: output");
        return 1;
    }
    int ok = fwrite(&lnl64, sizeof(double), 1, out) == 1 && fwrite(&lnl32, sizeof(double), 1, out) == 1 &&
             fwrite(&n_int, sizeof(int32_t), 1, out) == 1 && fwrite(nodes, sizeof(double), n_out, out) == n_out &&
             fwrite(sites, sizeof(double), n_sites, out) == (size_t)n_sites;
    ok = (fclose(out) == 0) && ok;
    free(masks); free(left); free(right); free(bl); free(Q); free(rw); free(cr); free(cw); free(nodes); free(sites);
    if (!ok) {
        fprintf(stderr, "plk_replay: write failed\n");
        return 1;
    }
    printf("lnL %.17g (FP64) %.17g (FP32S), %d internal nodes\n", lnl64, lnl32, (int)n_int);
    return 0;
}
