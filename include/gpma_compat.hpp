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
//
// The structure's members read as the reference's fields (gpma.cuh:31-50):
// gpma.keys, gpma.values and gpma.row_offset are views of the device arrays
// (data() gives the current device address, as RAW_PTR(gpma.keys) expects;
// size(); [i] copies one element to the host; to_host() the whole array);
// gpma.segment_length and gpma.tree_height convert to SIZE_TYPE and
// gpma.lower_element / gpma.upper_element to the threshold vectors, always
// for the current geometry (the array grows and shrinks with updates). Each
// of them can also be called, e.g. gpma.segment_length() or gpma.keys() for
// a host copy.
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

namespace detail {

inline gpma_geometry geometry_of(gpma_graph *h) {
    gpma_geometry g;
    check(gpma_get_geometry(h, &g), "GPMA::geometry");
    return g;
}

// A view of one device array of the structure (0 keys, 1 values, 2 row_offset).
template <typename T, int WHICH>
class DeviceArray {
  public:
    explicit DeviceArray(gpma_graph *const *h) : h_(h) {}
    T *data() const {
        const uint64_t *k = nullptr;
        const uint8_t *v = nullptr;
        const uint32_t *r = nullptr;
        check(gpma_device_arrays(*h_, &k, &v, &r), "GPMA device array");
        const void *p = WHICH == 0 ? (const void *)k : WHICH == 1 ? (const void *)v : (const void *)r;
        return static_cast<T *>(const_cast<void *>(p));
    }
    size_t size() const {
        const gpma_geometry g = geometry_of(*h_);
        return WHICH == 2 ? (size_t)g.row_num + 1 : (size_t)g.size;
    }
    std::vector<T> to_host() const {
        std::vector<T> out(size());
        void *dst[3] = {nullptr, nullptr, nullptr};
        dst[WHICH] = out.data();
        check(gpma_export_layout(*h_, static_cast<uint64_t *>(dst[0]), static_cast<uint8_t *>(dst[1]),
                                 static_cast<uint32_t *>(dst[2]), nullptr),
              "GPMA device array");
        return out;
    }
    std::vector<T> operator()() const { return to_host(); }
    T operator[](size_t i) const {
        const std::vector<T> all = to_host();
        if (i >= all.size())
            throw std::invalid_argument("GPMA device array: index out of range");
        return all[i];
    }

  private:
    gpma_graph *const *h_;
};

// segment_length / tree_height: the current geometry's value.
template <int WHICH>
class GeometryValue {
  public:
    explicit GeometryValue(gpma_graph *const *h) : h_(h) {}
    operator SIZE_TYPE() const {
        const gpma_geometry g = geometry_of(*h_);
        return WHICH == 0 ? g.segment_length : g.tree_height;
    }
    SIZE_TYPE operator()() const { return static_cast<SIZE_TYPE>(*this); }

  private:
    gpma_graph *const *h_;
};

// lower_element / upper_element: the current density thresholds per level.
template <int WHICH>
class Thresholds {
  public:
    explicit Thresholds(gpma_graph *const *h) : h_(h) {}
    std::vector<SIZE_TYPE> operator()() const {
        const SIZE_TYPE height = geometry_of(*h_).tree_height;
        std::vector<SIZE_TYPE> lo(height + 1), hi(height + 1);
        check(gpma_get_thresholds(*h_, lo.data(), hi.data()), "GPMA::thresholds");
        return WHICH == 0 ? lo : hi;
    }
    operator std::vector<SIZE_TYPE>() const { return (*this)(); }
    SIZE_TYPE operator[](size_t level) const {
        const std::vector<SIZE_TYPE> t = (*this)();
        if (level >= t.size())
            throw std::invalid_argument("GPMA thresholds: level out of range");
        return t[level];
    }
    size_t size() const { return (size_t)geometry_of(*h_).tree_height + 1; }

  private:
    gpma_graph *const *h_;
};

}  // namespace detail

template <dev_type_t DEV = GPU>
class GPMA {
    static_assert(DEV == GPU, "this library has no CPU structure: the update and BFS run on the GPU only");

  public:
    explicit GPMA(SIZE_TYPE row_num, void *stream = nullptr)
        : keys(&handle_), values(&handle_), row_offset(&handle_), segment_length(&handle_), tree_height(&handle_),
          lower_element(&handle_), upper_element(&handle_), row_num(row_num) {
        check(gpma_create(row_num, stream, &handle_), "GPMA(row_num)");
    }
    ~GPMA() { gpma_destroy(handle_); }
    GPMA(const GPMA &) = delete;
    GPMA &operator=(const GPMA &) = delete;

    int get_size() const { return (int)detail::geometry_of(handle_).size; }

    gpma_graph *handle() const { return handle_; }

  private:
    gpma_graph *handle_ = nullptr;  // declared before the views that refer to it

  public:
    // the reference's fields (gpma.cuh:31-50), read through the library
    const detail::DeviceArray<KEY_TYPE, 0> keys;
    const detail::DeviceArray<VALUE_TYPE, 1> values;
    const detail::DeviceArray<SIZE_TYPE, 2> row_offset;
    const detail::GeometryValue<0> segment_length;
    const detail::GeometryValue<1> tree_height;
    const detail::Thresholds<0> lower_element;
    const detail::Thresholds<1> upper_element;
    const SIZE_TYPE row_num;
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
