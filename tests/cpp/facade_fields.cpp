// The reference's field-style reads of a GPMA (gpma.cuh:31-50) against the
// facade: prints the geometry and checks that row_offset locates every row's
// guard key, reading keys and row_offset as the reference's device vectors.
#include "gpma_compat.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace gpma_compat;

int main(int argc, char **argv) {
    const SIZE_TYPE n = argc > 1 ? (SIZE_TYPE)std::atoi(argv[1]) : 64;
    GPMA<GPU> gpma(n);
    std::vector<KEY_TYPE> k;
    std::vector<VALUE_TYPE> v;
    for (SIZE_TYPE r = 0; r < n; ++r)
        for (SIZE_TYPE c = 0; c < (r % 7) + 1; ++c) {
            k.push_back(((KEY_TYPE)r << 32) + ((r * 13 + c * 5) % n));
            v.push_back(1);
        }
    update_gpma(gpma, k, v);
    const SIZE_TYPE seg = gpma.segment_length;  // fields, as in the reference
    const SIZE_TYPE height = gpma.tree_height;
    const std::vector<SIZE_TYPE> lower = gpma.lower_element;
    std::vector<KEY_TYPE> keys = gpma.keys.to_host();
    std::vector<SIZE_TYPE> ro = gpma.row_offset.to_host();
    int bad = 0;
    for (SIZE_TYPE r = 0; r < n; ++r)
        if (keys[ro[r + 1]] != (((KEY_TYPE)r << 32) | COL_IDX_NONE))
            ++bad;
    std::printf("size %zu seg %u height %u levels %zu upper_root %u guards_bad %d ptr %d first_guard_slot %u\n",
                gpma.keys.size(), seg, height, lower.size(), gpma.upper_element[height], bad,
                gpma.keys.data() != nullptr && gpma.row_offset.data() != nullptr, gpma.row_offset[1]);
    return bad == 0 && gpma.keys.size() == keys.size() && ro.size() == n + 1 && seg == gpma.segment_length() ? 0 : 1;
}
