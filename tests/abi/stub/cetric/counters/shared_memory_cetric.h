// TEST STAND-IN for KaTric's headers: just enough of the public types that
// include/katric_shim.hpp uses (DistributedGraph accessors, RankEncodedNodeId, Config,
// IntersectionMethod, profiling::Statistics), so the shim compiles and runs here as it would in
// a KaTric build.  Names and member signatures follow include/cetric/config.h:114,172-174,
// include/cetric/statistics.h:131-198, include/cetric/datastructures/graph_definitions.h:49-75
// and include/cetric/datastructures/distributed/distributed_graph.h:425-520,632-636 of the
// KaTric tree; the bodies are this test's own (one rank, no MPI).
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace cetric {

class RankEncodedNodeId {
public:
    RankEncodedNodeId() = default;
    RankEncodedNodeId(uint64_t id, uint16_t rank) : data_((uint64_t(rank) << 48) | id) {}
    uint64_t id() const { return data_ & ((uint64_t(1) << 48) - 1); }
    uint64_t data() const { return data_; }
    uint16_t rank() const { return uint16_t(data_ >> 48); }

private:
    uint64_t data_ = 0;
};

enum class IntersectionMethod { merge, binary_search, binary, hybrid };

struct Config {
    IntersectionMethod intersection_method = IntersectionMethod::merge;
    size_t binary_intersection_cutoff = 1000;
    double hybrid_cutoff_scale = 1.0;
};

namespace profiling {
struct Statistics {
    struct LocalStatistics {
        std::atomic<size_t> local_triangles{0};
    } local;
};
}  // namespace profiling

// One rank's graph.  Vertices 0..n_local-1 are local (rank 0); ids from n_local on are ghosts
// owned by rank 1.  Lists hold RankEncodedNodeIds.
template <class NodeIndexer = void>
class DistributedGraph {
public:
    struct Range {
        const RankEncodedNodeId* b;
        const RankEncodedNodeId* e;
        const RankEncodedNodeId* begin() const { return b; }
        const RankEncodedNodeId* end() const { return e; }
    };
    struct EdgeRange {
        Range r;
        Range neighbors() const { return r; }
    };

    // adj[v] (full lists) for every local vertex; out[v] the out-lists; ghost_out[g] the lists of
    // the ghosts (ids n_local + g)
    DistributedGraph(uint64_t n_local, std::vector<std::vector<uint64_t>> adj, std::vector<std::vector<uint64_t>> out,
                     std::vector<std::vector<uint64_t>> ghost_out)
        : n_local_(n_local) {
        auto enc = [&](const std::vector<std::vector<uint64_t>>& in, std::vector<std::vector<RankEncodedNodeId>>& to) {
            for (const auto& l : in) {
                to.emplace_back();
                for (uint64_t u : l) to.back().push_back(node(u));
            }
        };
        enc(adj, adj_);
        enc(out, out_);
        enc(ghost_out, ghost_);
        for (const auto& l : adj_) edges_ += l.size();
    }

    uint64_t local_node_count() const { return n_local_; }
    uint64_t local_edge_count() const { return edges_; }
    std::vector<RankEncodedNodeId> local_nodes() const {
        std::vector<RankEncodedNodeId> v;
        for (uint64_t i = 0; i < n_local_; ++i) v.push_back(node(i));
        return v;
    }
    std::vector<RankEncodedNodeId> ghosts() const {
        std::vector<RankEncodedNodeId> v;
        for (uint64_t g = 0; g < ghost_.size(); ++g) v.push_back(node(n_local_ + g));
        return v;
    }
    EdgeRange adj(RankEncodedNodeId v) const { return range(adj_[to_local_idx(v)]); }
    EdgeRange out_adj(RankEncodedNodeId v) const { return range(out_[to_local_idx(v)]); }
    EdgeRange ghost_adj(RankEncodedNodeId g) const { return range(ghost_[g.id() - n_local_]); }
    size_t to_local_idx(RankEncodedNodeId v) const { return size_t(v.id()); }
    size_t is_local(RankEncodedNodeId v) const { return v.rank() == 0; }

private:
    RankEncodedNodeId node(uint64_t i) const { return RankEncodedNodeId(i, i < n_local_ ? 0 : 1); }
    static EdgeRange range(const std::vector<RankEncodedNodeId>& l) { return {{l.data(), l.data() + l.size()}}; }
    uint64_t n_local_ = 0, edges_ = 0;
    std::vector<std::vector<RankEncodedNodeId>> adj_, out_, ghost_;
};

}  // namespace cetric
