// gpma_compat.hpp - C++ facade with the reference's API over the C ABI.
//
// Code written against recolic/gpma_bfs (gpma.cuh, gpma_bfs.cuh) switches by
// including this header instead and linking libgpma_gb300.so:
//
//   GPMA<GPU> gpma(node_size);                         // gpma.cuh:79-82
//   update_gpma(gpma, update_keys, update_values);     // gpma.cuh:968
//   gpma_bfs(gpma, node_size, edge_size, start, out);  // gpma_bfs.cuh:511-533
//
// Types are the reference's (utils.cuh:19-21): KEY_TYPE = uint64_t,
// VALUE_TYPE = char, SIZE_TYPE = uint32_t. update_gpma accepts any container
// with data()/size() (std::vector, thrust::host_vector, or
// thrust::device_vector through the overload enabled when Thrust is
// available); device or host memory is detected by the library. Unlike the
// reference, the batch is not modified. Errors throw: std::invalid_argument
// for mismatched key/value counts (as multidev.cuh:107-108) and bad
// arguments, std::runtime_error otherwise (the reference printed and went on,
// utils.cuh:56-61).
#pragma once

#include "gpma_gb300.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#if defined(__has_include)
#if __has_include(<thrust/device_vector.h>) && defined(__CUDACC__)
#include <thrust/device_vector.h>
#define GPMA_COMPAT_THRUST 1
#endif
#endif

namespace gpma_compat {

using KEY_TYPE = uint64_t;
using VALUE_TYPE = char;
using SIZE_TYPE = uint32_t;
constexpr KEY_TYPE KEY_NONE = (KEY_TYPE)(-1);        // gpma.cuh:15
constexpr KEY_TYPE KEY_MAX = KEY_NONE - 1;           // gpma.cuh:16
constexpr VALUE_TYPE VALUE_NONE = 0;                 // gpma.cuh:18
constexpr KEY_TYPE COL_IDX_NONE = 0xFFFFFFFF;        // gpma.cuh:19
enum dev_type_t : unsigned long { CPU = 19981223ul, GPU = 19990823ul };  // utils.cuh:27-28

inline void check(gpma_status s, const char *where) {
    if (s == GPMA_OK)
        return;
    std::string msg = std::string(where) + ": " + gpma_status_string(s) + ": " + gpma_last_error();
    if (s == GPMA_ERR_INVALID)
        throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

template <dev_type_t DEV = GPU>
class GPMA {
    static_assert(DEV == GPU, "this library has no CPU structure: the update and BFS run on the GPU only");

  public:
    explicit GPMA(SIZE_TYPE row_num, void *stream = nullptr) : row_num(row_num) {
        check(gpma_create(row_num, stream, &handle_), "GPMA(row_num)");
    }
    ~GPMA() { gpma_destroy(handle_); }
    GPMA(const GPMA &) = delete;
    GPMA &operator=(const GPMA &) = delete;

    int get_size() const { return (int)geometry().size; }
    SIZE_TYPE segment_length() const { return geometry().segment_length; }
    SIZE_TYPE tree_height() const { return geometry().tree_height; }
    std::vector<SIZE_TYPE> lower_element() const { return thresholds().first; }
    std::vector<SIZE_TYPE> upper_element() const { return thresholds().second; }

    // Host copies of the device arrays (GPMA::keys, values, row_offset).
    std::vector<KEY_TYPE> keys() const {
        std::vector<KEY_TYPE> k(geometry().size);
        check(gpma_export_layout(handle_, k.data(), nullptr, nullptr, nullptr), "GPMA::keys");
        return k;
    }
    std::vector<SIZE_TYPE> row_offset() const {
        std::vector<SIZE_TYPE> r((size_t)row_num + 1);
        check(gpma_export_layout(handle_, nullptr, nullptr, r.data(), nullptr), "GPMA::row_offset");
        return r;
    }

    gpma_graph *handle() const { return handle_; }
    const SIZE_TYPE row_num;

  private:
    gpma_geometry geometry() const {
        gpma_geometry g;
        check(gpma_get_geometry(handle_, &g), "GPMA::geometry");
        return g;
    }
    std::pair<std::vector<SIZE_TYPE>, std::vector<SIZE_TYPE>> thresholds() const {
        SIZE_TYPE h = tree_height();
        std::vector<SIZE_TYPE> lo(h + 1), hi(h + 1);
        check(gpma_get_thresholds(handle_, lo.data(), hi.data()), "GPMA::thresholds");
        return {lo, hi};
    }
    gpma_graph *handle_ = nullptr;
};

template <dev_type_t DEV>
void update_gpma(GPMA<DEV> &gpma, const KEY_TYPE *keys, const VALUE_TYPE *values, size_t n, void *stream = nullptr) {
    check(gpma_update(gpma.handle(), keys, reinterpret_cast<const uint8_t *>(values), n, stream), "update_gpma");
}

template <dev_type_t DEV, typename KeyVec, typename ValueVec>
void update_gpma(GPMA<DEV> &gpma, KeyVec &update_keys, ValueVec &update_values) {
    if (update_keys.size() != update_values.size())
        throw std::invalid_argument("Inconsistant kv size.");
    update_gpma(gpma, reinterpret_cast<const KEY_TYPE *>(update_keys.data()),
                reinterpret_cast<const VALUE_TYPE *>(update_values.data()), update_keys.size());
}

#ifdef GPMA_COMPAT_THRUST
template <dev_type_t DEV>
void update_gpma(GPMA<DEV> &gpma, thrust::device_vector<KEY_TYPE> &update_keys,
                 thrust::device_vector<VALUE_TYPE> &update_values) {
    if (update_keys.size() != update_values.size())
        throw std::invalid_argument("Inconsistant kv size.");
    update_gpma(gpma, thrust::raw_pointer_cast(update_keys.data()), thrust::raw_pointer_cast(update_values.data()),
                update_keys.size());
}
#endif

// results: node_size entries (host or device) of BFS levels, 1 at start_node,
// 0 where unreached. edge_size is accepted for signature parity (the
// reference sized its queues with it). Returns the reachable-node count.
template <dev_type_t DEV>
uint64_t gpma_bfs(GPMA<DEV> &gpma, SIZE_TYPE node_size, SIZE_TYPE edge_size, SIZE_TYPE start_node,
                  SIZE_TYPE *results, void *stream = nullptr) {
    (void)edge_size;
    if (node_size != gpma.row_num)
        throw std::invalid_argument("gpma_bfs: node_size differs from the structure's row_num");
    uint64_t reached = 0;
    check(::gpma_bfs(gpma.handle(), start_node, results, &reached, stream), "gpma_bfs");
    return reached;
}

}  // namespace gpma_compat
