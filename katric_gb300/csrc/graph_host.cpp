// Host-side graph ingest: seeded generators (G(n,m), RMAT, 2D RGG in Morton order),
// METIS and binary readers/writers, and the symmetrise/deduplicate/no-self-loop CSR
// builder.  Output is always a simple undirected graph in CSR form with u64 first_out
// and u32 head, every adjacency list sorted by id.
//
// Formats follow the reference's inputs:
//   - METIS text: header "n m [fmt]", then one 1-based adjacency line per vertex
//     (read by graph-io at apps/shmetric.cpp:119; sample files examples/*.metis).
//   - binary: <stem>.first_out = raw little-endian u64[n+1], <stem>.head = raw u64[2m],
//     0-based, both directions stored, no header (examples/*.first_out, examples/*.head).
// Generator output is deterministic for a given seed on every host and thread count:
// all randomness comes from a counter-based hash, lists are sorted before use, and
// floating-point distance tests are compiled without FMA contraction.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ktri.h"
#include "ktri_internal.h"

namespace {

// SplitMix64 finaliser as a counter-based generator: value = mix(key(seed, stream) + counter).
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t rng_at(uint64_t seed, uint64_t stream, uint64_t counter) {
    return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + counter * 0x9E3779B97F4A7C15ull);
}
// uniform in [0, n) by 64x64 -> high 64 multiply
inline uint64_t bounded(uint64_t r, uint64_t n) { return (uint64_t)(((unsigned __int128)r * n) >> 64); }
// uniform double in [0, 1) from the top 53 bits
inline double unit_double(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

ktri_graph* new_graph(uint64_t n, uint64_t nnz) {
    ktri_graph* g = new (std::nothrow) ktri_graph();
    if (!g) return nullptr;
    try {
        g->first_out.assign(n + 1, 0);
        g->head.resize(nnz);
    } catch (...) {
        delete g;
        return nullptr;
    }
    g->n = n;
    return g;
}

// Sort and deduplicate each adjacency list in place (lists live at [fo[v], fo[v]+cnt[v])),
// drop self-loops, then compact into a fresh CSR.
ktri_graph* finish_lists(uint64_t n, const std::vector<uint64_t>& fo, std::vector<uint32_t>& buf) {
    std::vector<uint64_t> deg(n);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t vi = 0; vi < (int64_t)n; ++vi) {
        uint64_t v = (uint64_t)vi;
        uint32_t* b = buf.data() + fo[v];
        uint32_t* e = buf.data() + fo[v + 1];
        std::sort(b, e);
        uint32_t* w = b;
        for (uint32_t* r = b; r != e; ++r) {
            if (*r == (uint32_t)v) continue;            // self-loop
            if (w != b && *(w - 1) == *r) continue;     // duplicate
            *w++ = *r;
        }
        deg[v] = (uint64_t)(w - b);
    }
    uint64_t nnz = 0;
    for (uint64_t v = 0; v < n; ++v) nnz += deg[v];
    ktri_graph* g = new_graph(n, nnz);
    if (!g) return nullptr;
    for (uint64_t v = 0; v < n; ++v) g->first_out[v + 1] = g->first_out[v] + deg[v];
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t vi = 0; vi < (int64_t)n; ++vi) {
        uint64_t v = (uint64_t)vi;
        std::memcpy(g->head.data() + g->first_out[v], buf.data() + fo[v], deg[v] * sizeof(uint32_t));
    }
    return g;
}

// Build a simple undirected CSR from an edge producer called twice (count, then fill).
// produce(i, &u, &v) returns false to skip sample i.  Both directions are inserted.
template <class Producer>
ktri_graph* build_from_samples(uint64_t n, uint64_t samples, Producer produce) {
    std::vector<std::atomic<uint64_t>> cnt(n);
    for (auto& c : cnt) c.store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static, 1 << 16)
    for (int64_t i = 0; i < (int64_t)samples; ++i) {
        uint32_t u, v;
        if (!produce((uint64_t)i, &u, &v) || u == v) continue;
        cnt[u].fetch_add(1, std::memory_order_relaxed);
        cnt[v].fetch_add(1, std::memory_order_relaxed);
    }
    std::vector<uint64_t> fo(n + 1, 0);
    for (uint64_t v = 0; v < n; ++v) fo[v + 1] = fo[v] + cnt[v].load(std::memory_order_relaxed);
    std::vector<uint32_t> buf(fo[n]);
    for (uint64_t v = 0; v < n; ++v) cnt[v].store(fo[v], std::memory_order_relaxed);
#pragma omp parallel for schedule(static, 1 << 16)
    for (int64_t i = 0; i < (int64_t)samples; ++i) {
        uint32_t u, v;
        if (!produce((uint64_t)i, &u, &v) || u == v) continue;
        buf[cnt[u].fetch_add(1, std::memory_order_relaxed)] = v;
        buf[cnt[v].fetch_add(1, std::memory_order_relaxed)] = u;
    }
    return finish_lists(n, fo, buf);
}

uint64_t morton_interleave16(uint32_t x, uint32_t y) {
    uint64_t r = 0;
    for (int b = 0; b < 32; ++b) {
        r |= (uint64_t)((x >> b) & 1u) << (2 * b);
        r |= (uint64_t)((y >> b) & 1u) << (2 * b + 1);
    }
    return r;
}

}  // namespace

extern "C" {

int ktri_graph_from_csr(uint64_t n, const uint64_t* first_out, const uint32_t* head, ktri_graph** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n > 0xFFFFFFFFull || !first_out || (n && first_out[0] != 0)) return KTRI_ERR_INVALID_CSR;
    uint64_t nnz = first_out[n];
    if (nnz && !head) return KTRI_ERR_INVALID_ARGUMENT;
    ktri_graph* g = new_graph(n, nnz);
    if (!g) return KTRI_ERR_OUT_OF_MEMORY;
    std::memcpy(g->first_out.data(), first_out, (n + 1) * sizeof(uint64_t));
    if (nnz) std::memcpy(g->head.data(), head, nnz * sizeof(uint32_t));
    *out = g;
    return KTRI_OK;
}

// G(n, m): m distinct undirected edges drawn uniformly without replacement, no self-loops.
// Candidates are drawn in counter order; the first m distinct ones are kept.
int ktri_graph_gnm(uint64_t n, uint64_t m, uint64_t seed, ktri_graph** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n < 2 || n > 0xFFFFFFFFull || m > n * (n - 1) / 2) return KTRI_ERR_INVALID_ARGUMENT;
    // open-addressing set of normalised edge keys (u << 32 | v, u < v)
    uint64_t cap = 1;
    while (cap < 2 * m + 16) cap <<= 1;
    std::vector<uint64_t> table(cap, ~0ull);
    std::vector<uint64_t> keys;
    keys.reserve(m);
    for (uint64_t i = 0; keys.size() < m; ++i) {
        uint64_t r = rng_at(seed, 1, i);
        uint64_t a = bounded(r, n), b = bounded(mix64(r), n);
        if (a == b) continue;
        uint64_t lo = std::min(a, b), hi = std::max(a, b);
        uint64_t k = (lo << 32) | hi;
        uint64_t h = mix64(k) & (cap - 1);
        bool seen = false;
        while (table[h] != ~0ull) {
            if (table[h] == k) { seen = true; break; }
            h = (h + 1) & (cap - 1);
        }
        if (seen) continue;
        table[h] = k;
        keys.push_back(k);
    }
    ktri_graph* g = build_from_samples(n, m, [&](uint64_t i, uint32_t* u, uint32_t* v) {
        *u = (uint32_t)(keys[i] >> 32);
        *v = (uint32_t)(keys[i] & 0xFFFFFFFFull);
        return true;
    });
    if (!g) return KTRI_ERR_OUT_OF_MEMORY;
    *out = g;
    return KTRI_OK;
}

// RMAT on n vertices: each of `samples` draws descends ceil(log2 n) levels choosing quadrant
// a (0,0), b (0,1), c (1,0) or d (1,1); draws that land outside [0, n)^2 are dropped.
// Symmetrised, deduplicated, self-loops removed, no vertex permutation.  For n = 2^scale this
// is the classic generator (nothing is dropped).
int ktri_graph_rmat_n(uint64_t n, uint64_t samples, double a, double b, double c, uint64_t seed, ktri_graph** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n < 2 || n > (1ull << 31) || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return KTRI_ERR_INVALID_ARGUMENT;
    uint32_t scale = 0;
    while ((1ull << scale) < n) ++scale;
    // 32-bit thresholds on a uniform 32-bit draw per level
    const double two32 = 4294967296.0;
    const uint64_t ta = (uint64_t)std::floor(a * two32);
    const uint64_t tb = (uint64_t)std::floor((a + b) * two32);
    const uint64_t tc = (uint64_t)std::floor((a + b + c) * two32);
    auto produce = [&](uint64_t i, uint32_t* u, uint32_t* v) {
        uint64_t x = 0, y = 0;
        uint64_t r = 0;
        for (uint32_t lvl = 0; lvl < scale; ++lvl) {
            if ((lvl & 1u) == 0) r = rng_at(seed, 2, i * 16 + lvl / 2);
            uint64_t p = (lvl & 1u) ? (r >> 32) : (r & 0xFFFFFFFFull);
            uint32_t bx, by;
            if (p < ta) { bx = 0; by = 0; }
            else if (p < tb) { bx = 0; by = 1; }
            else if (p < tc) { bx = 1; by = 0; }
            else { bx = 1; by = 1; }
            x = (x << 1) | bx;
            y = (y << 1) | by;
        }
        if (x >= n || y >= n) return false;
        *u = (uint32_t)x;
        *v = (uint32_t)y;
        return true;
    };
    ktri_graph* g = build_from_samples(n, samples, produce);
    if (!g) return KTRI_ERR_OUT_OF_MEMORY;
    *out = g;
    return KTRI_OK;
}

// RMAT: 2^scale vertices, edge_factor * 2^scale samples.
int ktri_graph_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                    ktri_graph** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (scale < 1 || scale > 31) return KTRI_ERR_INVALID_ARGUMENT;
    return ktri_graph_rmat_n(1ull << scale, (uint64_t)edge_factor << scale, a, b, c, seed, out);
}

// 2D random geometric graph: n points uniform in [0,1)^2, edge iff squared distance < r^2,
// r = sqrt(avg_degree / (pi n)).  Vertex ids are the rank of each point in Morton order of
// its coordinates quantised to 2^16 cells per axis (ties broken by draw index).
int ktri_graph_rgg2d(uint64_t n, double avg_degree, uint64_t seed, ktri_graph** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n < 1 || n > 0xFFFFFFFFull || !(avg_degree >= 0)) return KTRI_ERR_INVALID_ARGUMENT;
    const double r = std::sqrt(avg_degree / (M_PI * (double)n));
    const double r2 = r * r;
    std::vector<double> px(n), py(n);
    std::vector<uint64_t> order(n);
    std::vector<std::pair<uint64_t, uint64_t>> codes(n);
#pragma omp parallel for schedule(static, 1 << 14)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        double x = unit_double(rng_at(seed, 3, 2 * (uint64_t)i));
        double y = unit_double(rng_at(seed, 3, 2 * (uint64_t)i + 1));
        uint32_t qx = (uint32_t)std::min(65535.0, std::floor(x * 65536.0));
        uint32_t qy = (uint32_t)std::min(65535.0, std::floor(y * 65536.0));
        codes[i] = {morton_interleave16(qx, qy), (uint64_t)i};
        px[i] = x;
        py[i] = y;
    }
    std::sort(codes.begin(), codes.end());
    std::vector<double> X(n), Y(n);
    for (uint64_t k = 0; k < n; ++k) {
        X[k] = px[codes[k].second];
        Y[k] = py[codes[k].second];
    }
    px.clear(); px.shrink_to_fit();
    py.clear(); py.shrink_to_fit();
    codes.clear(); codes.shrink_to_fit();
    // uniform grid with cell side >= r
    uint64_t G = r > 0 ? (uint64_t)std::floor(1.0 / r) : 1;
    if (G < 1) G = 1;
    if (G > 65536) G = 65536;
    auto cell_of = [&](double v) { uint64_t c = (uint64_t)(v * (double)G); return c >= G ? G - 1 : c; };
    std::vector<uint64_t> cell_start(G * G + 1, 0);
    std::vector<uint64_t> cell_id(n);
    for (uint64_t k = 0; k < n; ++k) {
        cell_id[k] = cell_of(Y[k]) * G + cell_of(X[k]);
        cell_start[cell_id[k] + 1]++;
    }
    for (uint64_t c = 0; c < G * G; ++c) cell_start[c + 1] += cell_start[c];
    std::vector<uint32_t> cell_pts(n);
    {
        std::vector<uint64_t> cur(cell_start.begin(), cell_start.end() - 1);
        for (uint64_t k = 0; k < n; ++k) cell_pts[cur[cell_id[k]]++] = (uint32_t)k;
    }
    auto visit = [&](uint64_t k, auto&& fn) {
        int64_t cx = (int64_t)cell_of(X[k]), cy = (int64_t)cell_of(Y[k]);
        for (int64_t dy = -1; dy <= 1; ++dy)
            for (int64_t dx = -1; dx <= 1; ++dx) {
                int64_t x = cx + dx, y = cy + dy;
                if (x < 0 || y < 0 || x >= (int64_t)G || y >= (int64_t)G) continue;
                uint64_t c = (uint64_t)y * G + (uint64_t)x;
                for (uint64_t p = cell_start[c]; p < cell_start[c + 1]; ++p) {
                    uint32_t j = cell_pts[p];
                    if (j == k) continue;
                    double ddx = X[k] - X[j], ddy = Y[k] - Y[j];
                    double d2 = ddx * ddx + ddy * ddy;
                    if (d2 < r2) fn(j);
                }
            }
    };
    std::vector<uint64_t> deg(n);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        uint64_t c = 0;
        visit((uint64_t)k, [&](uint32_t) { ++c; });
        deg[k] = c;
    }
    uint64_t nnz = 0;
    for (uint64_t k = 0; k < n; ++k) nnz += deg[k];
    ktri_graph* g = new_graph(n, nnz);
    if (!g) return KTRI_ERR_OUT_OF_MEMORY;
    for (uint64_t k = 0; k < n; ++k) g->first_out[k + 1] = g->first_out[k] + deg[k];
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        uint32_t* w = g->head.data() + g->first_out[k];
        uint32_t* b = w;
        visit((uint64_t)k, [&](uint32_t j) { *w++ = j; });
        std::sort(b, w);
    }
    *out = g;
    return KTRI_OK;
}

// METIS text reader: header "n m [fmt]" (fmt must be 0 or absent: no weights), then one
// 1-based adjacency line per vertex; '%' lines are comments.  Adjacency order is kept.
int ktri_graph_read_metis(const char* path, ktri_graph** out) {
    if (!out || !path) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return KTRI_ERR_IO;
    std::string data;
    {
        char buf[1 << 16];
        size_t k;
        while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) data.append(buf, k);
        std::fclose(f);
    }
    size_t pos = 0;
    auto next_line = [&](std::string& line) -> bool {
        while (pos < data.size()) {
            size_t e = data.find('\n', pos);
            if (e == std::string::npos) e = data.size();
            line.assign(data, pos, e - pos);
            pos = e + 1;
            if (!line.empty() && line[0] == '%') continue;
            return true;
        }
        return false;
    };
    std::string line;
    if (!next_line(line)) return KTRI_ERR_IO;
    unsigned long long n = 0, m = 0, fmt = 0;
    int k = std::sscanf(line.c_str(), "%llu %llu %llu", &n, &m, &fmt);
    if (k < 2 || fmt != 0 || n > 0xFFFFFFFFull) return KTRI_ERR_IO;
    ktri_graph* g = new_graph(n, 0);
    if (!g) return KTRI_ERR_OUT_OF_MEMORY;
    g->head.reserve(2 * m);
    for (uint64_t v = 0; v < n; ++v) {
        if (!next_line(line)) line.clear();
        const char* s = line.c_str();
        char* end;
        while (true) {
            while (*s == ' ' || *s == '\t' || *s == '\r') ++s;
            if (!*s) break;
            unsigned long long x = std::strtoull(s, &end, 10);
            if (end == s || x < 1 || x > n) { delete g; return KTRI_ERR_IO; }
            g->head.push_back((uint32_t)(x - 1));
            s = end;
        }
        g->first_out[v + 1] = g->head.size();
    }
    if (g->head.size() != 2 * m) { delete g; return KTRI_ERR_IO; }
    *out = g;
    return KTRI_OK;
}

// Binary reader: <stem>.first_out (u64[n+1]) and <stem>.head (u64[nnz]), little-endian.
int ktri_graph_read_binary(const char* stem, ktri_graph** out) {
    if (!out || !stem) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::string s(stem);
    auto slurp = [](const std::string& p, std::vector<uint64_t>& v) -> bool {
        FILE* f = std::fopen(p.c_str(), "rb");
        if (!f) return false;
        std::fseek(f, 0, SEEK_END);
        long sz = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (sz < 0 || sz % 8) { std::fclose(f); return false; }
        v.resize((size_t)sz / 8);
        size_t got = v.empty() ? 0 : std::fread(v.data(), 8, v.size(), f);
        std::fclose(f);
        return got == v.size();
    };
    std::vector<uint64_t> fo, hd;
    if (!slurp(s + ".first_out", fo) || !slurp(s + ".head", hd) || fo.empty()) return KTRI_ERR_IO;
    uint64_t n = fo.size() - 1;
    if (n > 0xFFFFFFFFull || fo[0] != 0 || fo[n] != hd.size()) return KTRI_ERR_INVALID_CSR;
    for (uint64_t v = 0; v < n; ++v)
        if (fo[v + 1] < fo[v]) return KTRI_ERR_INVALID_CSR;
    ktri_graph* g = new_graph(n, hd.size());
    if (!g) return KTRI_ERR_OUT_OF_MEMORY;
    g->first_out = fo;
    for (size_t i = 0; i < hd.size(); ++i) {
        if (hd[i] >= n) { delete g; return KTRI_ERR_INVALID_CSR; }
        g->head[i] = (uint32_t)hd[i];
    }
    *out = g;
    return KTRI_OK;
}

// Binary writer in the reference's input format (u64 heads), so that the reference's
// `shmetric --input-format binary` reads the identical graph.
int ktri_graph_write_binary(const ktri_graph* g, const char* stem) {
    if (!g || !stem) return KTRI_ERR_INVALID_ARGUMENT;
    std::string s(stem);
    FILE* f = std::fopen((s + ".first_out").c_str(), "wb");
    if (!f) return KTRI_ERR_IO;
    bool ok = std::fwrite(g->first_out.data(), 8, g->first_out.size(), f) == g->first_out.size();
    std::fclose(f);
    if (!ok) return KTRI_ERR_IO;
    f = std::fopen((s + ".head").c_str(), "wb");
    if (!f) return KTRI_ERR_IO;
    std::vector<uint64_t> chunk(1 << 16);
    for (size_t i = 0; i < g->head.size() && ok; i += chunk.size()) {
        size_t k = std::min(chunk.size(), g->head.size() - i);
        for (size_t j = 0; j < k; ++j) chunk[j] = g->head[i + j];
        ok = std::fwrite(chunk.data(), 8, k, f) == k;
    }
    std::fclose(f);
    return ok ? KTRI_OK : KTRI_ERR_IO;
}

int ktri_graph_write_metis(const ktri_graph* g, const char* path) {
    if (!g || !path) return KTRI_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return KTRI_ERR_IO;
    std::fprintf(f, "%llu %llu\n", (unsigned long long)g->n, (unsigned long long)(g->head.size() / 2));
    for (uint64_t v = 0; v < g->n; ++v) {
        for (uint64_t e = g->first_out[v]; e < g->first_out[v + 1]; ++e)
            std::fprintf(f, e == g->first_out[v] ? "%u" : " %u", g->head[e] + 1);
        std::fputc('\n', f);
    }
    bool ok = std::fclose(f) == 0;
    return ok ? KTRI_OK : KTRI_ERR_IO;
}

// Disjoint union of graphs: graph k's vertices become [graph_first[k], graph_first[k+1]).
static ktri_graph* pack_union(const std::vector<ktri_graph*>& gs, uint64_t* graph_first) {
    const size_t k = gs.size();
    std::vector<uint64_t> nnz_first(k + 1, 0);
    graph_first[0] = 0;
    for (size_t i = 0; i < k; ++i) {
        graph_first[i + 1] = graph_first[i] + gs[i]->n;
        nnz_first[i + 1] = nnz_first[i] + gs[i]->head.size();
    }
    if (graph_first[k] > 0xFFFFFFFFull) return nullptr;
    ktri_graph* u = new_graph(graph_first[k], nnz_first[k]);
    if (!u) return nullptr;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ii = 0; ii < (int64_t)k; ++ii) {
        const ktri_graph* g = gs[(size_t)ii];
        const uint64_t vb = graph_first[ii], eb = nnz_first[ii];
        for (uint64_t v = 0; v < g->n; ++v) u->first_out[vb + v + 1] = eb + g->first_out[v + 1];
        for (uint64_t e = 0; e < g->head.size(); ++e) u->head[eb + e] = (uint32_t)(g->head[e] + vb);
    }
    return u;
}

int ktri_batch_pack(uint64_t num_graphs, const ktri_graph* const* graphs, ktri_graph** out, uint64_t* graph_first) {
    if (!out || !graph_first || (num_graphs && !graphs)) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::vector<ktri_graph*> gs(num_graphs);
    for (uint64_t i = 0; i < num_graphs; ++i) {
        if (!graphs[i]) return KTRI_ERR_INVALID_ARGUMENT;
        gs[i] = const_cast<ktri_graph*>(graphs[i]);
    }
    ktri_graph* u = pack_union(gs, graph_first);
    if (!u) return graph_first[num_graphs] > 0xFFFFFFFFull ? KTRI_ERR_UNSUPPORTED : KTRI_ERR_OUT_OF_MEMORY;
    *out = u;
    return KTRI_OK;
}

// A batch of independent graphs: graph i has n_i = round(2^U(log2_n_min, log2_n_max))
// vertices and average degree d_i = U(deg_min, deg_max); generator i mod 3 picks G(n,m)
// (m = round(n d / 2)), RMAT (0.57, 0.19, 0.19, 0.05) with round(n d / 2) draws, or the 2D
// RGG; graph i is seeded with seed + i.  Graphs are generated in parallel, one per thread.
int ktri_batch_generate(uint64_t num_graphs, double log2_n_min, double log2_n_max, double deg_min, double deg_max,
                        uint64_t seed, ktri_graph** out, uint64_t* graph_first) {
    if (!out || !graph_first) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!(log2_n_min >= 1) || log2_n_max < log2_n_min || log2_n_max > 31 || !(deg_min >= 0) || deg_max < deg_min)
        return KTRI_ERR_INVALID_ARGUMENT;
    std::vector<ktri_graph*> gs(num_graphs, nullptr);
    std::atomic<int> rc{KTRI_OK};
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ii = 0; ii < (int64_t)num_graphs; ++ii) {
        const uint64_t i = (uint64_t)ii;
        const double u1 = unit_double(rng_at(seed, 4, 2 * i)), u2 = unit_double(rng_at(seed, 4, 2 * i + 1));
        uint64_t n = (uint64_t)std::llround(std::exp2(log2_n_min + (log2_n_max - log2_n_min) * u1));
        if (n < 2) n = 2;
        const double d = deg_min + (deg_max - deg_min) * u2;
        const uint64_t half = (uint64_t)std::llround((double)n * d / 2.0);
        int r;
        switch (i % 3) {
            case 0: r = ktri_graph_gnm(n, std::min(half, n * (n - 1) / 2), seed + i, &gs[i]); break;
            case 1: r = ktri_graph_rmat_n(n, half, 0.57, 0.19, 0.19, seed + i, &gs[i]); break;
            default: r = ktri_graph_rgg2d(n, d, seed + i, &gs[i]); break;
        }
        if (r != KTRI_OK) rc.store(r);
    }
    int result = rc.load();
    if (result == KTRI_OK) {
        ktri_graph* u = pack_union(gs, graph_first);
        if (!u) result = graph_first[num_graphs] > 0xFFFFFFFFull ? KTRI_ERR_UNSUPPORTED : KTRI_ERR_OUT_OF_MEMORY;
        else *out = u;
    }
    for (ktri_graph* g : gs) delete g;
    return result;
}

// Many graphs from explicit specs, generated in parallel (one thread per graph): graph i is
// kinds[i] = 0 G(n,m) with m = round(n d / 2), 1 RMAT with round(n d / 2) draws, 2 2D RGG
// with average degree d; n = ns[i], d = degrees[i], seed = seeds[i].
int ktri_graphs_generate(uint64_t count, const uint32_t* kinds, const uint64_t* ns, const double* degrees,
                         const uint64_t* seeds, ktri_graph** outs) {
    if (!outs || (count && (!kinds || !ns || !degrees || !seeds))) return KTRI_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < count; ++i) outs[i] = nullptr;
    std::atomic<int> rc{KTRI_OK};
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ii = 0; ii < (int64_t)count; ++ii) {
        const uint64_t i = (uint64_t)ii, n = ns[i];
        const double d = degrees[i];
        const uint64_t half = (uint64_t)std::llround((double)n * d / 2.0);
        int r;
        switch (kinds[i]) {
            case 0: r = ktri_graph_gnm(n, std::min(half, n * (n - 1) / 2), seeds[i], &outs[i]); break;
            case 1: r = ktri_graph_rmat_n(n, half, 0.57, 0.19, 0.19, seeds[i], &outs[i]); break;
            case 2: r = ktri_graph_rgg2d(n, d, seeds[i], &outs[i]); break;
            default: r = KTRI_ERR_INVALID_ARGUMENT;
        }
        if (r != KTRI_OK) rc.store(r);
    }
    if (rc.load() != KTRI_OK) {
        for (uint64_t i = 0; i < count; ++i) {
            delete outs[i];
            outs[i] = nullptr;
        }
    }
    return rc.load();
}

uint64_t ktri_graph_n(const ktri_graph* g) { return g ? g->n : 0; }
uint64_t ktri_graph_nnz(const ktri_graph* g) { return g ? g->head.size() : 0; }
const uint64_t* ktri_graph_first_out(const ktri_graph* g) { return g ? g->first_out.data() : nullptr; }
const uint32_t* ktri_graph_head(const ktri_graph* g) { return g ? g->head.data() : nullptr; }
void ktri_graph_free(ktri_graph* g) { delete g; }

}  // extern "C"
