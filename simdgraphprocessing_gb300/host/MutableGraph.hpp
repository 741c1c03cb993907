// Drop-in MutableGraph (the reference's src/MutableGraph.hpp:49-93): the same
// public fields and static loaders, backed by the engine's host graph
// (eh_hgraph_*).  Undirected graphs only (the pattern-count path).
#ifndef EH_DROPIN_MUTABLEGRAPH_HPP
#define EH_DROPIN_MUTABLEGRAPH_HPP

#include "common.hpp"

struct MutableGraph {
  size_t num_nodes;
  size_t num_edges;
  size_t max_nbrhood_size;
  bool symmetric;
  vector<uint64_t>* id_map;
  vector<uint32_t>* node_attr;
  vector<vector<uint32_t>*>* out_neighborhoods;
  vector<vector<uint32_t>*>* in_neighborhoods;
  vector<vector<uint32_t>*>* out_edge_attributes;
  vector<vector<uint32_t>*>* in_edge_attributes;

  MutableGraph(size_t num_nodes_in, size_t num_edges_in, size_t max_nbrhood_size_in, bool symmetric_in,
               vector<uint64_t>* id_map_in, vector<uint32_t>* node_attr_in,
               vector<vector<uint32_t>*>* out_neighborhoods_in, vector<vector<uint32_t>*>* in_neighborhoods_in,
               vector<vector<uint32_t>*>* out_edge_attributes_in, vector<vector<uint32_t>*>* in_edge_attributes_in)
      : num_nodes(num_nodes_in),
        num_edges(num_edges_in),
        max_nbrhood_size(max_nbrhood_size_in),
        symmetric(symmetric_in),
        id_map(id_map_in),
        node_attr(node_attr_in),
        out_neighborhoods(out_neighborhoods_in),
        in_neighborhoods(in_neighborhoods_in),
        out_edge_attributes(out_edge_attributes_in),
        in_edge_attributes(in_edge_attributes_in) {}

  ~MutableGraph() {
    if (out_neighborhoods) {
      for (auto* r : *out_neighborhoods) delete r;
      delete out_neighborhoods;
    }
    delete id_map;
  }

  // CSR view of the adjacency (rows must be sorted ascending).
  void to_csr(vector<uint64_t>& offsets, vector<uint32_t>& nbrs) const {
    offsets.assign(num_nodes + 1, 0);
    for (size_t i = 0; i < num_nodes; i++) offsets[i + 1] = offsets[i] + out_neighborhoods->at(i)->size();
    nbrs.resize(offsets[num_nodes]);
    for (size_t i = 0; i < num_nodes; i++) {
      const vector<uint32_t>* r = out_neighborhoods->at(i);
      if (!r->empty()) std::memcpy(&nbrs[offsets[i]], r->data(), r->size() * sizeof(uint32_t));
    }
  }

  static MutableGraph* from_hgraph(eh_hgraph_t h) {
    uint64_t n = 0, m = 0, mx = 0;
    const uint64_t* off = nullptr;
    const uint32_t* nbr = nullptr;
    const uint64_t* ext = nullptr;
    common::check(eh_hgraph_view(h, &n, &m, &off, &nbr, &ext, &mx));
    auto* ids = new vector<uint64_t>(ext, ext + n);
    auto* rows = new vector<vector<uint32_t>*>(n);
    for (uint64_t i = 0; i < n; i++) (*rows)[i] = new vector<uint32_t>(nbr + off[i], nbr + off[i + 1]);
    eh_hgraph_free(h);
    return new MutableGraph(n, m, mx, true, ids, nullptr, rows, rows, nullptr, nullptr);
  }

  eh_hgraph_t to_hgraph() const {
    vector<uint64_t> off;
    vector<uint32_t> nbr;
    to_csr(off, nbr);
    eh_hgraph_t h = nullptr;
    common::check(eh_hgraph_from_csr(num_nodes, off.data(), nbr.data(), id_map->data(), &h));
    return h;
  }

  // MutableGraph::undirectedFromBinary (src/MutableGraph.hpp:316-360).
  static MutableGraph* undirectedFromBinary(const string path) {
    eh_hgraph_t h = nullptr;
    common::check(eh_hgraph_read_binary(path.c_str(), &h));
    return from_hgraph(h);
  }
  // MutableGraph::undirectedFromEdgeList (src/MutableGraph.hpp:517-599).
  static MutableGraph* undirectedFromEdgeList(const string path) {
    eh_hgraph_t h = nullptr;
    common::check(eh_hgraph_read_edge_list(path.c_str(), &h));
    return from_hgraph(h);
  }
  // MutableGraph::writeUndirectedToBinary (src/MutableGraph.hpp:298-314).
  void writeUndirectedToBinary(const string path) {
    eh_hgraph_t h = to_hgraph();
    eh_status s = eh_hgraph_write_binary(h, path.c_str());
    eh_hgraph_free(h);
    common::check(s);
  }
  // MutableGraph::reorder_by_degree (src/MutableGraph.hpp:268-272).
  void reorder_by_degree() {
    eh_hgraph_t h = to_hgraph();
    common::check(eh_hgraph_reorder_by_degree(h));
    MutableGraph* g = from_hgraph(h);
    for (auto* r : *out_neighborhoods) delete r;
    delete out_neighborhoods;
    delete id_map;
    out_neighborhoods = in_neighborhoods = g->out_neighborhoods;
    id_map = g->id_map;
    g->out_neighborhoods = g->in_neighborhoods = nullptr;
    g->id_map = nullptr;
    delete g;
  }
};

#endif
