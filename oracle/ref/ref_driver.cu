// Runs a GPMA workload script through the reference implementation itself:
// `GPMA<CPU>` + `update_gpma<CPU>` (gpma.cuh:31-102, 968-1050) and the
// reference's CPU BFS gather/contract pair (gpma_bfs.cuh:397-443) driven by the
// same level loop as gpma_bfs_multidev_single (gpma_bfs.cuh:446-509).
//
// This binary is test infrastructure: it produces the golden vectors that pin
// the C restatement in oracle/gpma_oracle.c. It is built from the reference
// sources in place by oracle/Makefile (target `ref`) into oracle/_ref/.
//
// Script format (little endian), shared with oracle/workload.py:
//   "GPWS" u32 version(=1) u32 row_num u32 n_ops, then n_ops records:
//     u32 op=1 (update): u64 n, u64 keys[n], u8 values[n]
//     u32 op=2 (bfs):    u32 src
//     u32 op=3 (dump):   no payload; writes the full layout
// Output format: "GPWO" u32 version(=1), then one record per op:
//     op=1: u32 tag=1, u32 size, seg, height, row_num, u64 live, u64 digest[4]
//           (layout keys, masked values, row_offset, compacted live keys),
//           u32 lower[height+1], u32 upper[height+1]
//     op=2: u32 tag=2, u32 src, u64 reached, u32 levels[row_num]
//     op=3: u32 tag=3, u32 size, u32 row_num, u64 keys[size],
//           u8 masked_values[size], u32 row_offset[row_num+1]
// cpu_alg.hpp throws std::runtime_error without including <stdexcept>.
#include <stdexcept>

#include "gpma.cuh"
#include "gpma_bfs.cuh"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Order-sensitive digest of a sequence of unsigned integers (each widened to
// 64 bits); identical to digest() in oracle/workload.py.
template <typename T>
uint64_t digest(const T *x, size_t n) {
    uint64_t acc = 0;
    for (size_t i = 0; i < n; ++i)
        acc += mix64((uint64_t)x[i] + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull);
    return acc;
}

void die(const char *msg) {
    std::fprintf(stderr, "ref_driver: %s\n", msg);
    std::exit(2);
}

template <typename T>
void rd(FILE *f, T *p, size_t n) {
    if (n && std::fread(p, sizeof(T), n, f) != n)
        die("short read");
}
template <typename T>
void wr(FILE *f, const T *p, size_t n) {
    if (n && std::fwrite(p, sizeof(T), n, f) != n)
        die("short write");
}

struct State {
    std::vector<uint64_t> keys;
    std::vector<uint8_t> masked;
    std::vector<uint32_t> row_offset;
};

State snapshot(GPMA<CPU> &g) {
    State s;
    size_t size = g.keys.size();
    s.keys.assign(g.keys.begin(), g.keys.end());
    s.masked.resize(size);
    for (size_t i = 0; i < size; ++i)
        s.masked[i] = (s.keys[i] == KEY_NONE) ? 0 : (uint8_t)g.values[i];
    s.row_offset.assign(g.row_offset.begin(), g.row_offset.end());
    return s;
}

void run_bfs(GPMA<CPU> &g, uint32_t n, uint32_t src, std::vector<uint32_t> &results) {
    // Mirrors gpma_bfs_multidev_single<CPU> with one CPU instance and no GPU.
    results.assign(n, 0);
    std::vector<uint32_t> bitmap(n / 32 + 2, 0);
    std::vector<uint32_t> node_q(3 * (size_t)n + 3, 0);
    std::vector<uint32_t> edge_q(g.keys.size() + 1, 0);
    uint32_t node_q_size = 0, edge_q_size = 0;
    node_q[0] = src;
    bitmap[src / 32] = 1u << (src % 32);
    node_q_size = 1;
    results[src] = 1;
    uint32_t level = 1;
    while (true) {
        edge_q_size = 0;
        gpma_bfs_gather_cpu(node_q.data(), &node_q_size, edge_q.data(), &edge_q_size, RAW_PTR(g.keys), RAW_PTR(g.values),
                            RAW_PTR(g.row_offset));
        node_q_size = 0;
        level++;
        gpma_bfs_contract_cpu(edge_q.data(), &edge_q_size, node_q.data(), &node_q_size, level, results.data(), bitmap.data());
        if (node_q_size == 0)
            break;
    }
}

} // namespace

int main(int argc, char **argv) {
    if (argc != 3)
        die("usage: ref_driver <script.gws> <out.gwo>");
    FILE *in = std::fopen(argv[1], "rb");
    if (!in)
        die("cannot open script");
    FILE *out = std::fopen(argv[2], "wb");
    if (!out)
        die("cannot open output");
    char magic[4];
    rd(in, magic, 4);
    if (std::memcmp(magic, "GPWS", 4) != 0)
        die("bad magic");
    uint32_t version, row_num, n_ops;
    rd(in, &version, 1);
    rd(in, &row_num, 1);
    rd(in, &n_ops, 1);
    if (version != 1)
        die("bad version");
    wr(out, "GPWO", 4);
    wr(out, &version, 1);

    GPMA<CPU> g(row_num);
    for (uint32_t op_i = 0; op_i < n_ops; ++op_i) {
        uint32_t op;
        rd(in, &op, 1);
        if (op == 1) {
            uint64_t n;
            rd(in, &n, 1);
            std::vector<uint64_t> k(n);
            std::vector<uint8_t> v(n);
            rd(in, k.data(), n);
            rd(in, v.data(), n);
            NATIVE_VEC_KEY<CPU> uk(k.begin(), k.end());
            NATIVE_VEC_VALUE<CPU> uv(n);
            for (uint64_t i = 0; i < n; ++i)
                uv[i] = (VALUE_TYPE)v[i];
            update_gpma(g, uk, uv);
            State s = snapshot(g);
            std::vector<uint64_t> compact;
            for (size_t i = 0; i < s.keys.size(); ++i)
                if (s.keys[i] != KEY_NONE && g.values[i] != VALUE_NONE)
                    compact.push_back(s.keys[i]);
            uint32_t tag = 1, size = (uint32_t)s.keys.size(), seg = g.segment_length, h = g.tree_height;
            uint64_t live = compact.size();
            uint64_t d[4] = {digest(s.keys.data(), s.keys.size()), digest(s.masked.data(), s.masked.size()),
                             digest(s.row_offset.data(), s.row_offset.size()), digest(compact.data(), compact.size())};
            wr(out, &tag, 1);
            wr(out, &size, 1);
            wr(out, &seg, 1);
            wr(out, &h, 1);
            wr(out, &row_num, 1);
            wr(out, &live, 1);
            wr(out, d, 4);
            std::vector<uint32_t> lo(g.lower_element.begin(), g.lower_element.end());
            std::vector<uint32_t> hi(g.upper_element.begin(), g.upper_element.end());
            wr(out, lo.data(), lo.size());
            wr(out, hi.data(), hi.size());
        } else if (op == 4) {
            // timed update: update_gpma alone, its wall time in nanoseconds
            // (no layout digest), for timing the reference's CPU path
            uint64_t n;
            rd(in, &n, 1);
            std::vector<uint64_t> k(n);
            std::vector<uint8_t> v(n);
            rd(in, k.data(), n);
            rd(in, v.data(), n);
            NATIVE_VEC_KEY<CPU> uk(k.begin(), k.end());
            NATIVE_VEC_VALUE<CPU> uv(n);
            for (uint64_t i = 0; i < n; ++i)
                uv[i] = (VALUE_TYPE)v[i];
            const auto t0 = std::chrono::steady_clock::now();
            update_gpma(g, uk, uv);
            const uint64_t ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                                    std::chrono::steady_clock::now() - t0)
                                    .count();
            uint32_t tag = 4;
            wr(out, &tag, 1);
            wr(out, &n, 1);
            wr(out, &ns, 1);
        } else if (op == 2) {
            uint32_t src;
            rd(in, &src, 1);
            if (src >= row_num)
                die("bfs source out of range");
            std::vector<uint32_t> levels;
            run_bfs(g, row_num, src, levels);
            uint64_t reached = 0;
            for (uint32_t x : levels)
                reached += (x != 0);
            uint32_t tag = 2;
            wr(out, &tag, 1);
            wr(out, &src, 1);
            wr(out, &reached, 1);
            wr(out, levels.data(), levels.size());
        } else if (op == 3) {
            State s = snapshot(g);
            uint32_t tag = 3, size = (uint32_t)s.keys.size();
            wr(out, &tag, 1);
            wr(out, &size, 1);
            wr(out, &row_num, 1);
            wr(out, s.keys.data(), s.keys.size());
            wr(out, s.masked.data(), s.masked.size());
            wr(out, s.row_offset.data(), s.row_offset.size());
        } else {
            die("unknown op");
        }
    }
    std::fclose(out);
    std::fclose(in);
    return 0;
}
