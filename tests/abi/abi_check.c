/* TEST PROGRAM: include/ktri.h as a C compiler sees it.
 *
 *   abi_check sizes                 print sizeof / offsetof of the ABI structs (no CUDA call)
 *   abi_check count <stem>...       read each <stem>.first_out/.head (the reference's binary graph
 *                                   format) with ktri_graph_read_binary and count it through
 *                                   ktri_count_csr and ktri_count_csr_ctx; print
 *                                   "<stem> <total> <total_ctx> <sum of per-vertex>"
 * Exit status 0 on success. */
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ktri.h"

#define FIELD(T, f) printf("%s.%s %zu %zu\n", #T, #f, offsetof(T, f), sizeof(((T*)0)->f))

static int sizes(void) {
    printf("ktri_opts %zu\n", sizeof(ktri_opts));
    FIELD(ktri_opts, struct_size);
    FIELD(ktri_opts, intersection_method);
    FIELD(ktri_opts, small_outdegree);
    FIELD(ktri_opts, collect_stats);
    FIELD(ktri_opts, binary_intersection_cutoff);
    FIELD(ktri_opts, hybrid_cutoff_scale);
    FIELD(ktri_opts, force_wide_offsets);
    FIELD(ktri_opts, medium_outdegree);
    FIELD(ktri_opts, segment);
    FIELD(ktri_opts, copy_wait_polls);
    FIELD(ktri_opts, tile_order);
    FIELD(ktri_opts, reserved);
    printf("ktri_run_stats %zu\n", sizeof(ktri_run_stats));
    FIELD(ktri_run_stats, triangles);
    FIELD(ktri_run_stats, n);
    FIELD(ktri_run_stats, nnz);
    FIELD(ktri_run_stats, oriented_edges);
    FIELD(ktri_run_stats, wedge_checks);
    FIELD(ktri_run_stats, intersection_size_local);
    FIELD(ktri_run_stats, streamed_entries);
    FIELD(ktri_run_stats, input_sorted);
    FIELD(ktri_run_stats, method);
    FIELD(ktri_run_stats, ms_orient);
    FIELD(ktri_run_stats, ms_count);
    FIELD(ktri_run_stats, ms_total);
    FIELD(ktri_run_stats, ms_count_small);
    FIELD(ktri_run_stats, ms_count_large);
    FIELD(ktri_run_stats, ms_h2d);
    FIELD(ktri_run_stats, ms_d2h);
    FIELD(ktri_run_stats, ms_call);
    FIELD(ktri_run_stats, host_ms_enqueue);
    FIELD(ktri_run_stats, host_ms_call);
    FIELD(ktri_run_stats, streamed_chunked);
    printf("ktri_server_opts %zu\n", sizeof(ktri_server_opts));
    FIELD(ktri_server_opts, struct_size);
    FIELD(ktri_server_opts, slots);
    FIELD(ktri_server_opts, memory_budget);
    FIELD(ktri_server_opts, max_batch_nnz);
    FIELD(ktri_server_opts, max_batch_graphs);
    FIELD(ktri_server_opts, direct_host_access);
    FIELD(ktri_server_opts, engine);
    FIELD(ktri_server_opts, reserved);
    printf("ktri_server_stats %zu\n", sizeof(ktri_server_stats));
    FIELD(ktri_server_stats, submitted);
    FIELD(ktri_server_stats, coalesced);
    FIELD(ktri_server_stats, device_us);
    FIELD(ktri_server_stats, engine_launches);
    FIELD(ktri_server_stats, reserved);
    printf("ktri_tuning %zu\n", sizeof(ktri_tuning));
    FIELD(ktri_tuning, intersection_method);
    FIELD(ktri_tuning, candidates);
    FIELD(ktri_tuning, tile_order);
    FIELD(ktri_tuning, ms);
    FIELD(ktri_tuning, default_ms);
    FIELD(ktri_tuning, signature);
    return 0;
}

static int count(int argc, char** argv) {
    ktri_ctx* ctx = NULL;
    int rc = ktri_ctx_create(0, &ctx);
    if (rc != KTRI_OK) {
        fprintf(stderr, "ktri_ctx_create: %d\n", rc);
        return 1;
    }
    for (int i = 0; i < argc; ++i) {
        ktri_graph* g = NULL;
        rc = ktri_graph_read_binary(argv[i], &g);
        if (rc != KTRI_OK) {
            fprintf(stderr, "read %s: %d\n", argv[i], rc);
            return 1;
        }
        const uint64_t n = ktri_graph_n(g), nnz = ktri_graph_nnz(g);
        uint64_t* pv = (uint64_t*)calloc(n ? n : 1, sizeof(uint64_t));
        uint64_t t1 = 0, t2 = 0, sum = 0;
        ktri_opts opts;
        memset(&opts, 0, sizeof opts);
        opts.struct_size = sizeof opts;
        opts.intersection_method = KTRI_METHOD_AUTO;
        rc = ktri_count_csr(ktri_graph_first_out(g), ktri_graph_head(g), n, nnz, &t1, NULL, NULL);
        if (rc == KTRI_OK)
            rc = ktri_count_csr_ctx(ctx, ktri_graph_first_out(g), ktri_graph_head(g), n, nnz, &t2, pv, &opts);
        if (rc != KTRI_OK) {
            fprintf(stderr, "count %s: %d (%s)\n", argv[i], rc, ktri_last_error(ctx));
            return 1;
        }
        for (uint64_t v = 0; v < n; ++v) sum += pv[v];
        printf("%s %llu %llu %llu\n", argv[i], (unsigned long long)t1, (unsigned long long)t2,
               (unsigned long long)sum);
        free(pv);
        ktri_graph_free(g);
    }
    ktri_ctx_destroy(ctx);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && strcmp(argv[1], "sizes") == 0) return sizes();
    if (argc >= 3 && strcmp(argv[1], "count") == 0) return count(argc - 2, argv + 2);
    fprintf(stderr, "usage: abi_check sizes | count <stem>...\n");
    return 2;
}
