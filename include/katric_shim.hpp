// katric_shim.hpp: KaTric's counting entry points on the GPU engine (C ABI in ktri.h).
//
// For a KaTric build: include this header after cetric/counters/shared_memory_cetric.h (it
// includes that header itself) and link with -lktri.  It only reads the graph through
// DistributedGraph's public accessors and leaves it untouched (the reference orients and
// sorts G in place).
//
//   run_shmem_gpu  replaces size_t cetric::run_shmem(DistributedGraph<>&, Statistics&, const Config&)
//                  (include/cetric/counters/shared_memory_cetric.h:105, called from apps/shmetric.cpp:140):
//                  preprocessing + run_local + combine, one exact total, optional per-vertex counts.
//   run_local_gpu  replaces CetricEdgeIterator::run_local on one rank's oriented lists, ghosts
//                  included (include/cetric/counters/cetric_edge_iterator.h:230-388, called from
//                  include/cetric/cetric.h:431,450,827,847), where its emit callback only counts.
//
// Both throw std::runtime_error on a non-zero status, as the reference throws on its own
// errors (include/cetric/util.h:105-117); no exception crosses the C ABI itself.
#pragma once

#include <ktri.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "cetric/counters/shared_memory_cetric.h"

namespace cetric {

// The hot-path fields of cetric::Config (include/cetric/config.h:172-174) as ktri_opts.
inline ktri_opts ktri_opts_from(const Config& conf) {
    ktri_opts opts{};
    opts.struct_size = sizeof(ktri_opts);
    switch (conf.intersection_method) {  // --intersection-method keeps its meaning
        case IntersectionMethod::merge: opts.intersection_method = KTRI_METHOD_MERGE; break;
        case IntersectionMethod::binary_search: opts.intersection_method = KTRI_METHOD_BINARY_SEARCH; break;
        case IntersectionMethod::binary: opts.intersection_method = KTRI_METHOD_BINARY; break;
        case IntersectionMethod::hybrid: opts.intersection_method = KTRI_METHOD_HYBRID; break;
    }
    opts.binary_intersection_cutoff = conf.binary_intersection_cutoff;
    opts.hybrid_cutoff_scale = conf.hybrid_cutoff_scale;
    return opts;
}

// run_shmem on the GPU.  The local vertices become ids 0..n-1 (to_local_idx); the rank bits of
// every RankEncodedNodeId are stripped with .id().  With use_auto the engine's owner-side hash
// kernels run (the fast default); otherwise the configured reference strategy does.  Both give
// the same count.
template <typename Graph>
size_t run_shmem_gpu(Graph& G, profiling::Statistics& stats, const Config& conf,
                     std::vector<uint64_t>* per_vertex = nullptr, bool use_auto = true) {
    const uint64_t n = G.local_node_count();
    std::vector<uint64_t> first_out(n + 1, 0);
    std::vector<uint32_t> head;
    head.reserve(G.local_edge_count());
    for (auto v : G.local_nodes()) {
        for (auto u : G.adj(v).neighbors()) head.push_back(static_cast<uint32_t>(u.id()));
        first_out[G.to_local_idx(v) + 1] = head.size();
    }
    ktri_opts opts = ktri_opts_from(conf);
    if (use_auto) opts.intersection_method = KTRI_METHOD_AUTO;
    uint64_t total = 0;
    if (per_vertex) per_vertex->assign(n, 0);
    const int rc = ktri_count_csr(first_out.data(), head.data(), n, head.size(), &total,
                                  per_vertex ? per_vertex->data() : nullptr, &opts);
    if (rc != KTRI_OK) throw std::runtime_error("ktri_count_csr failed with status " + std::to_string(rc));
    stats.local.local_triangles += total;
    return total;
}

// run_local on the GPU for one rank: local vertices first (to_local_idx), then the ghosts in
// the order G.ghosts() gives them.  Every edge must sit in exactly one of the lists, as after
// the reference's preprocessing (out_adj of local vertices, ghost_adj of ghosts).
template <typename Graph>
size_t run_local_gpu(const Graph& G, profiling::Statistics& stats, ktri_ctx* ctx,
                     std::vector<uint64_t>* per_vertex = nullptr) {
    const uint64_t nl = G.local_node_count();
    std::unordered_map<uint64_t, uint32_t> ghost_idx;
    for (auto g : G.ghosts()) ghost_idx.emplace(g.data(), static_cast<uint32_t>(nl + ghost_idx.size()));
    auto index = [&](auto u) -> uint32_t {
        return G.is_local(u) ? static_cast<uint32_t>(G.to_local_idx(u)) : ghost_idx.at(u.data());
    };
    const uint64_t n = nl + ghost_idx.size();
    std::vector<std::vector<uint32_t>> lists(n);
    for (auto v : G.local_nodes())
        for (auto u : G.out_adj(v).neighbors()) lists[G.to_local_idx(v)].push_back(index(u));
    for (auto g : G.ghosts())
        for (auto u : G.ghost_adj(g).neighbors()) lists[ghost_idx.at(g.data())].push_back(index(u));
    std::vector<uint64_t> first_out(n + 1, 0);
    std::vector<uint32_t> head;
    for (uint64_t i = 0; i < n; ++i) {
        head.insert(head.end(), lists[i].begin(), lists[i].end());
        first_out[i + 1] = head.size();
    }
    uint64_t total = 0;
    if (per_vertex) per_vertex->assign(n, 0);
    const int rc = ktri_count_dag_ctx(ctx, first_out.data(), head.data(), n, head.size(), &total,
                                      per_vertex ? per_vertex->data() : nullptr, nullptr);
    if (rc != KTRI_OK) throw std::runtime_error(ktri_last_error(ctx));
    stats.local.local_triangles += total;
    return total;
}

}  // namespace cetric
