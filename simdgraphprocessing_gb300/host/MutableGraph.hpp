// Drop-in MutableGraph (the reference's src/MutableGraph.hpp:49-93): the same
// public fields and static loaders, backed by the engine's host graph
// (eh_hgraph_*).  Undirected graphs share one neighbourhood list for out and
// in; directed graphs (symmetric == false) keep both.
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
    if (in_neighborhoods && in_neighborhoods != out_neighborhoods) {
      for (auto* r : *in_neighborhoods) delete r;
      delete in_neighborhoods;
    }
    if (out_neighborhoods) {
      for (auto* r : *out_neighborhoods) delete r;
      delete out_neighborhoods;
    }
    delete id_map;
  }

  // CSR view of a neighbourhood list (rows must be sorted ascending).
  static void rows_to_csr(const vector<vector<uint32_t>*>* rows, size_t n, vector<uint64_t>& offsets,
                          vector<uint32_t>& nbrs) {
    offsets.assign(n + 1, 0);
    for (size_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + rows->at(i)->size();
    nbrs.resize(offsets[n]);
    for (size_t i = 0; i < n; i++) {
      const vector<uint32_t>* r = rows->at(i);
      if (!r->empty()) std::memcpy(&nbrs[offsets[i]], r->data(), r->size() * sizeof(uint32_t));
    }
  }
  // The out-neighbourhoods (the rows) as CSR.
  void to_csr(vector<uint64_t>& offsets, vector<uint32_t>& nbrs) const {
    rows_to_csr(out_neighborhoods, num_nodes, offsets, nbrs);
  }
  // The in-neighbourhoods (the columns) as CSR.
  void to_in_csr(vector<uint64_t>& offsets, vector<uint32_t>& nbrs) const {
    rows_to_csr(in_neighborhoods, num_nodes, offsets, nbrs);
  }

  static vector<vector<uint32_t>*>* rows_of(uint64_t n, const uint64_t* off, const uint32_t* nbr) {
    auto* rows = new vector<vector<uint32_t>*>(n);
    for (uint64_t i = 0; i < n; i++) (*rows)[i] = new vector<uint32_t>(nbr + off[i], nbr + off[i + 1]);
    return rows;
  }

  static MutableGraph* from_hgraph(eh_hgraph_t h) {
    uint64_t n = 0, m = 0, mx = 0, in_m = 0;
    const uint64_t* off = nullptr;
    const uint32_t* nbr = nullptr;
    const uint64_t* ext = nullptr;
    const uint64_t* ioff = nullptr;
    const uint32_t* inbr = nullptr;
    int directed = 0;
    common::check(eh_hgraph_view(h, &n, &m, &off, &nbr, &ext, &mx));
    common::check(eh_hgraph_in_view(h, &directed, &in_m, &ioff, &inbr));
    auto* ids = new vector<uint64_t>(ext, ext + n);
    auto* rows = rows_of(n, off, nbr);
    auto* cols = directed ? rows_of(n, ioff, inbr) : rows;
    eh_hgraph_free(h);
    // The reference's directed loaders count out and in entries (MutableGraph.hpp:675-688).
    return new MutableGraph(n, directed ? m + in_m : m, mx, !directed, ids, nullptr, rows, cols, nullptr, nullptr);
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
  // MutableGraph::directedFromBinary (src/MutableGraph.hpp:656-714).
  static MutableGraph* directedFromBinary(const string path) {
    eh_hgraph_t h = nullptr;
    common::check(eh_hgraph_read_directed_binary(path.c_str(), &h));
    return from_hgraph(h);
  }
  // MutableGraph::directedFromEdgeList (src/MutableGraph.hpp:893-986).
  static MutableGraph* directedFromEdgeList(const string path) {
    eh_hgraph_t h = nullptr;
    common::check(eh_hgraph_read_directed_edge_list(path.c_str(), &h));
    return from_hgraph(h);
  }
  // MutableGraph::writeDirectedToBinary (src/MutableGraph.hpp:634-654): per node
  // u64 external id, size_t out length, out ids, size_t in length, in ids.
  void writeDirectedToBinary(const string path) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot open " + path + " for writing");
    bool ok = fwrite(&num_nodes, sizeof(size_t), 1, f) == 1;
    for (size_t i = 0; i < num_nodes && ok; i++) {
      ok = fwrite(&id_map->at(i), sizeof(uint64_t), 1, f) == 1;
      for (const vector<uint32_t>* r : {out_neighborhoods->at(i), in_neighborhoods->at(i)}) {
        const size_t len = r->size();
        ok = ok && fwrite(&len, sizeof(size_t), 1, f) == 1;
        if (ok && len) ok = fwrite(r->data(), sizeof(uint32_t), len, f) == len;
      }
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) throw std::runtime_error("write to " + path + " failed");
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
