// The reference demo's flow (gpma_bfs_demo.cu:32-116) written against the
// drop-in facade: load "n m" + m edge lines, insert the first half, BFS,
// slide 100 times (next step edges in, oldest step edges out), BFS again.
#include "gpma_compat.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace gpma_compat;

int main(int argc, char **argv) {
    if (argc != 3) {
        std::printf("Invalid arguments.\n");
        return -1;
    }
    FILE *fp = std::fopen(argv[1], "r");
    if (!fp) {
        std::printf("Open graph file failed.\n");
        return 1;
    }
    int bfs_start_node = std::atoi(argv[2]);
    int node_size = 0, edge_size = 0;
    if (std::fscanf(fp, "%d %d", &node_size, &edge_size) != 2)
        return 1;
    std::printf("node_num: %d, edge_num: %d\n", node_size, edge_size);
    std::vector<int> host_x(edge_size), host_y(edge_size);
    for (int i = 0; i < edge_size; i++)
        if (std::fscanf(fp, "%d %d", &host_x[i], &host_y[i]) != 2)
            return 1;
    std::fclose(fp);
    std::printf("Graph file is loaded.\n");

    int half = edge_size / 2;
    std::vector<KEY_TYPE> base_keys(half);
    for (int i = 0; i < half; i++)
        base_keys[i] = ((KEY_TYPE)host_x[i] << 32) + host_y[i];
    std::vector<VALUE_TYPE> base_values(half, 1);
    int num_slide = 100;
    int step = half / num_slide;

    GPMA<GPU> gpma(node_size);
    update_gpma(gpma, base_keys, base_values);
    std::vector<SIZE_TYPE> bfs_result(node_size);
    uint64_t reach = gpma_bfs(gpma, node_size, edge_size, bfs_start_node, bfs_result.data());
    std::printf("start from node %d, number of reachable nodes: %llu\n", bfs_start_node, (unsigned long long)reach);

    for (int i = 0; i < num_slide; i++) {
        std::vector<KEY_TYPE> hk(step * 2);
        for (int j = 0; j < step; j++) {
            int idx = half + i * step + j;
            hk[j] = ((KEY_TYPE)host_x[idx] << 32) + host_y[idx];
        }
        for (int j = 0; j < step; j++) {
            int idx = i * step + j;
            hk[j + step] = ((KEY_TYPE)host_x[idx] << 32) + host_y[idx];
        }
        std::vector<VALUE_TYPE> update_values(step * 2, VALUE_NONE);
        for (int j = 0; j < step; j++)
            update_values[j] = 1;
        update_gpma(gpma, hk, update_values);
    }
    std::printf("Graph is updated.\n");
    reach = gpma_bfs(gpma, node_size, edge_size, bfs_start_node, bfs_result.data());
    std::printf("start from node %d, number of reachable nodes: %llu\n", bfs_start_node, (unsigned long long)reach);
    return 0;
}
