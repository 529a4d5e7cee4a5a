// Test driver of simit_gb300::Map (simit_gb300/cpp/map.h): builds facade
// Sets from a text description, runs one user map whose element function
// source is read from a file, and writes the pattern and values.
//
// Input (whitespace separated):
//   <source file> <bs> <vector 0|1> <fp64 0|1>
//   <n vertices> <card, 0 = a map over the vertices> <n elements>
//   <endpoints: elements x card ints>
//   <n fields>, then per field: <element|vertex> <name> <f64|i32|b8> <comps> <values>
// Output: "rowptr" line, "colidx" line, "values" line (%.17g).
#include <cstdio>
#include <fstream>
#include <sstream>

#include "simit_gb300/cpp/simit.h"

using namespace simit_gb300;

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: map_driver INPUT OUTPUT\n");
    return 2;
  }
  try {
    std::ifstream in(argv[1]);
    std::string srcpath;
    int bs, vec, fp64, n, card, nE;
    in >> srcpath >> bs >> vec >> fp64 >> n >> card >> nE;
    std::ifstream sf(srcpath);
    std::stringstream ss;
    ss << sf.rdbuf();
    Set V;
    std::unique_ptr<Set> E = card ? Set::edge_set(card) : nullptr;
    std::vector<int32_t> ep((size_t)nE * card);
    for (auto &v : ep) in >> v;
    int nf;
    in >> nf;
    struct Pending {
      bool elem;
      std::string name, type;
      int comps;
      std::vector<double> vals;
    };
    std::vector<Pending> fs(nf);
    std::vector<std::string> order;
    for (auto &f : fs) {
      std::string kind;
      in >> kind >> f.name >> f.type >> f.comps;
      f.elem = kind == "element";
      const int count = (f.elem ? (card ? nE : n) : n) * f.comps;
      f.vals.resize(count);
      for (auto &x : f.vals) in >> x;
      order.push_back((f.elem ? "element:" : "vertex:") + f.name);
    }
    if (!in) throw SimitException("map_driver: truncated input");
    // fields first, then elements (add() grows every field)
    for (auto &f : fs) {
      Set &s = (f.elem && card) ? *E : V;
      s.add_field_raw(f.name,
                      f.type == "i32" ? FieldType::I32
                                      : (f.type == "b8" ? FieldType::BOOL : FieldType::F64),
                      f.comps);
    }
    for (int i = 0; i < n; ++i) V.add();
    if (card)
      for (int e = 0; e < nE; ++e) E->add_with_endpoints(ep.data() + (size_t)e * card);
    for (auto &f : fs) {
      Set &s = (f.elem && card) ? *E : V;
      FieldData *d = s.field(f.name);
      for (size_t i = 0; i < f.vals.size(); ++i) {
        if (f.type == "i32") reinterpret_cast<int32_t *>(d->data.data())[i] = (int32_t)f.vals[i];
        else if (f.type == "b8") reinterpret_cast<bool *>(d->data.data())[i] = f.vals[i] != 0;
        else reinterpret_cast<double *>(d->data.data())[i] = f.vals[i];
      }
    }
    Map m(ss.str(), bs, vec != 0, order, fp64 != 0);
    m.bind(card ? E.get() : &V, &V);
    m.runSafe();
    std::FILE *o = std::fopen(argv[2], "w");
    if (!o) throw SimitException("map_driver: cannot write the output");
    std::fprintf(o, "rowptr");
    for (uint32_t r : m.rowptr()) std::fprintf(o, " %u", r);
    std::fprintf(o, "\ncolidx");
    for (uint32_t c : m.colidx()) std::fprintf(o, " %u", c);
    std::fprintf(o, "\nvalues");
    for (double v : m.values()) std::fprintf(o, " %.17g", v);
    std::fprintf(o, "\n");
    std::fclose(o);
  } catch (const std::exception &e) {
    std::printf("FAIL exception: %s\n", e.what());
    return 1;
  }
  std::printf("map_driver ok\n");
  return 0;
}
