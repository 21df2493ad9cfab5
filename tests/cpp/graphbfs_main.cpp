// A driver in the shape of the reference's 1D Partition/main.cu:10-82,
// written against include/gbfs_graphbfs.hpp.
// usage: graphbfs <input_file> <source_num>; prints the time line and the
// level array (one value per line).
#include <cstdio>
#include <string>

#include "gbfs_graphbfs.hpp"

int main(int argc, char *argv[])
{
    if (argc != 3) {
        std::cerr << "Usage: " << argv[0] << " <input_file> <source_num>" << std::endl;
        return 1;
    }
    try {
        gbfs::csr graph(argv[1]);
        gbfs::gpuBFS bfs(graph, std::stoi(argv[2]));
        std::cout << "GPU BFS Time: " << bfs.exec_time << " ms" << std::endl;
        for (int i = 0; i < graph.num_nodes; i++) std::printf("%d\n", bfs.host_distance[i]);
    } catch (const gbfs::error &e) {
        std::cerr << e.what() << std::endl;
        return 2;
    }
    return 0;
}
