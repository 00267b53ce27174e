// TEST PROGRAM: include/katric_shim.hpp compiled against a stand-in of KaTric's types
// (tests/abi/stub), as a KaTric build would compile it.
//
//   shim_check sizes            print sizeof(ktri_opts) and sizeof(ktri_run_stats) as C++ sees them
//   shim_check count <stem>     read <stem>.first_out/.head; count it with cetric::run_shmem_gpu
//                               (AUTO and the configured merge strategy), then with
//                               cetric::run_local_gpu on two "ranks" of the same graph (vertices
//                               split in half, the second half as ghosts of the first); print
//                               "<total_auto> <total_merge> <sum_per_vertex> <local_rank0>"
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "katric_shim.hpp"

int main(int argc, char** argv) {
    if (argc >= 2 && std::strcmp(argv[1], "sizes") == 0) {
        std::printf("ktri_opts %zu\nktri_run_stats %zu\n", sizeof(ktri_opts), sizeof(ktri_run_stats));
        return 0;
    }
    if (argc < 3 || std::strcmp(argv[1], "count") != 0) {
        std::fprintf(stderr, "usage: shim_check sizes | count <stem>\n");
        return 2;
    }
    ktri_graph* g = nullptr;
    if (ktri_graph_read_binary(argv[2], &g) != KTRI_OK) return 1;
    const uint64_t n = ktri_graph_n(g);
    const uint64_t* fo = ktri_graph_first_out(g);
    const uint32_t* hd = ktri_graph_head(g);
    std::vector<std::vector<uint64_t>> adj(n), out(n);
    for (uint64_t v = 0; v < n; ++v)
        for (uint64_t e = fo[v]; e < fo[v + 1]; ++e) {
            adj[v].push_back(hd[e]);
            if (hd[e] > v) out[v].push_back(hd[e]);  // any orientation works for run_local_gpu
        }
    try {
        cetric::profiling::Statistics stats;
        cetric::Config conf;  // merge, as the reference defaults
        cetric::DistributedGraph<> G(n, adj, out, {});
        std::vector<uint64_t> pv;
        const size_t t_auto = cetric::run_shmem_gpu(G, stats, conf, &pv);
        const size_t t_merge = cetric::run_shmem_gpu(G, stats, conf, nullptr, false);
        uint64_t sum = 0;
        for (uint64_t c : pv) sum += c;
        // rank 0 of a two-rank split: local vertices [0, h) keep their out-lists (higher ids,
        // ghosts among them); the ghosts [h, n) bring their own out-lists, which hold the edges
        // between ghosts.  Every edge then sits in exactly one list, so the count is the total.
        const uint64_t h = n / 2;
        std::vector<std::vector<uint64_t>> ladj(adj.begin(), adj.begin() + h), lout(out.begin(), out.begin() + h),
            gout(out.begin() + h, out.end());
        cetric::DistributedGraph<> L(h, ladj, lout, gout);
        ktri_ctx* ctx = nullptr;
        if (ktri_ctx_create(0, &ctx) != KTRI_OK) return 1;
        cetric::profiling::Statistics lstats;
        const size_t t_local = cetric::run_local_gpu(L, lstats, ctx);
        ktri_ctx_destroy(ctx);
        std::printf("%zu %zu %llu %zu\n", t_auto, t_merge, (unsigned long long)sum, t_local);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "shim: %s\n", e.what());
        return 1;
    }
    ktri_graph_free(g);
    return 0;
}
