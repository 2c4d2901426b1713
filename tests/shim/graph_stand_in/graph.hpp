// A minimal stand-in for the reference's Graph (src/graph.hpp), for hosts
// without the reference sources: only the members the shim reads, the
// constructor the shim's driver calls, and ownership of the two CSR arrays.
#ifndef GRAPH_HPP
#define GRAPH_HPP

#include <cstddef>

class Graph {
   public:
    const int n;
    const int m;
    const int *const indices;
    const int *const adj;

    Graph(int num_nodes, int num_edges, int *adj_, int *indices_, int *, int *, int * = NULL)
        : n(num_nodes), m(num_edges), indices(indices_), adj(adj_) {}
    ~Graph() {
        delete[] indices;
        delete[] adj;
    }
};

#endif
