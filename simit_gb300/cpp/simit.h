// C++ host facade of simit_gb300 with the reference's user API for the
// sparse-system path: simit::Set / ElementRef / FieldRef
// (src/graph.h:91-749) and simit::Function's bind / init / run / runSafe /
// mapArgs / unmapArgs (src/function.h:30-95).  There is no DSL compiler
// behind Function: it runs one of the built-in programs of the path, each the
// GPU version of a reference .sim program:
//
//   "isprings"      test/input/program/isprings.sim  main
//   "isprings_app"  apps/springs/isprings.sim        timestep
//   "cg"            test/input/program/cg.sim        main
//   "femTet"        test/input/program/femTet.sim    main   (+ "femTet.init" = initializeTet)
//
// Field names and meanings are the .sim programs' own.  Errors from the C
// ABI become SimitException, as simit_uassert raises it (src/error.cpp:86-97).
// Header-only; link with libsimit_gb300.so and libcudart.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/simit_gb300.h"

namespace simit_gb300 {

class SimitException : public std::runtime_error {
 public:
  explicit SimitException(const std::string &m) : std::runtime_error(m) {}
};

inline void check(int rc, const char *what) {
  if (rc != SG_OK)
    throw SimitException(std::string(what) + ": " + sg_last_error());
}
inline void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw SimitException(std::string(what) + ": " + cudaGetErrorString(e));
}

struct ElementRef {
  int ident = -1;
  bool defined() const { return ident >= 0; }
};

enum class FieldType { F64, F32, I32, BOOL };

struct FieldData {
  std::string name;
  FieldType type;
  int comps;                       // product of the field's dimensions
  std::vector<unsigned char> data; // SoA: element-major, comps values each
  size_t elem_size() const {
    return type == FieldType::F64 ? 8 : (type == FieldType::BOOL ? 1 : 4);
  }
};

template <typename T> struct FieldTypeOf;
template <> struct FieldTypeOf<double> { static constexpr FieldType v = FieldType::F64; };
template <> struct FieldTypeOf<float> { static constexpr FieldType v = FieldType::F32; };
template <> struct FieldTypeOf<int> { static constexpr FieldType v = FieldType::I32; };
template <> struct FieldTypeOf<bool> { static constexpr FieldType v = FieldType::BOOL; };

class Set;

// FieldRef<T, dims...>: typed handle to one field of a set.
template <typename T, int... dims> class FieldRef {
 public:
  static constexpr int kComps = (1 * ... * dims);
  FieldRef() = default;
  FieldRef(Set *s, int idx) : set_(s), idx_(idx) {}
  T *ptr(ElementRef e) const;
  // x(p)(i): component i of element p
  struct Acc {
    T *p;
    T &operator()(int i) const { return p[i]; }
    T &operator[](int i) const { return p[i]; }
    Acc &operator=(std::initializer_list<T> v) {
      int i = 0;
      for (T t : v) p[i++] = t;
      return *this;
    }
    operator T() const { return p[0]; }
    Acc &operator=(T v) {
      p[0] = v;
      return *this;
    }
  };
  Acc operator()(ElementRef e) const { return Acc{ptr(e)}; }
  Acc get(ElementRef e) const { return Acc{ptr(e)}; }
  void set(ElementRef e, std::initializer_list<T> v) const { Acc{ptr(e)} = v; }
  void set(ElementRef e, T v) const { *ptr(e) = v; }

 private:
  Set *set_ = nullptr;
  int idx_ = -1;
};

// Set: a vertex set (no endpoints) or an edge set with `card` endpoints in
// other sets; fields are SoA arrays that grow with add().
class Set {
 public:
  Set() = default;
  template <typename... S> explicit Set(S &...endpoint_sets) : card_(sizeof...(S)) {
    endpoint_sets_ = {&endpoint_sets...};
  }
  Set(const Set &) = delete;
  Set &operator=(const Set &) = delete;

  template <typename T, int... dims> FieldRef<T, dims...> addField(const std::string &name) {
    FieldData f{name, FieldTypeOf<T>::v, FieldRef<T, dims...>::kComps, {}};
    f.data.resize(size_ * f.comps * f.elem_size());
    fields_.push_back(std::move(f));
    return FieldRef<T, dims...>(this, (int)fields_.size() - 1);
  }

  // A field whose type is known at run time (comps values per element).
  FieldData &add_field_raw(const std::string &name, FieldType type, int comps) {
    FieldData f{name, type, comps, {}};
    f.data.resize(size_ * f.comps * f.elem_size());
    fields_.push_back(std::move(f));
    return fields_.back();
  }

  ElementRef add() {
    if (card_ != 0) throw SimitException("Set::add: edge sets take endpoints");
    return grow();
  }
  template <typename... E> ElementRef add(E... eps) {
    if ((int)sizeof...(E) != card_) throw SimitException("Set::add: wrong number of endpoints");
    ElementRef r = grow();
    for (ElementRef e : {eps...}) endpoints_.push_back(e.ident);
    return r;
  }

  // An element whose card endpoints are given as an array.
  ElementRef add_with_endpoints(const int32_t *eps) {
    ElementRef r = grow();
    for (int k = 0; k < card_; ++k) endpoints_.push_back(eps[k]);
    return r;
  }
  // An edge set over sets that are not facade Sets (card endpoints each).
  static std::unique_ptr<Set> edge_set(int card) {
    std::unique_ptr<Set> s(new Set());
    s->card_ = card;
    return s;
  }

  int getSize() const { return size_; }
  int numFields() const { return (int)fields_.size(); }
  int getCardinality() const { return card_; }
  const std::vector<int32_t> &endpoints() const { return endpoints_; }
  int32_t *getEndpointsPtr() { return endpoints_.data(); }
  std::vector<FieldData> &getFields() { return fields_; }

  // The field holding the elements' positions, which reorder() sorts along a
  // Hilbert curve (src/graph.h: setSpatialField / hasSpatialField).
  void setSpatialField(const std::string &name) {
    if (!field(name)) throw SimitException("Set::setSpatialField: no field " + name);
    spatial_ = name;
  }
  bool hasSpatialField() const { return !spatial_.empty(); }
  const std::string &getSpatialFieldName() const { return spatial_; }
  FieldData *field(const std::string &name) {
    for (auto &f : fields_)
      if (f.name == name) return &f;
    return nullptr;
  }
  FieldData &field_at(int i) { return fields_[i]; }

 private:
  ElementRef grow() {
    for (auto &f : fields_) f.data.resize((size_ + 1) * f.comps * f.elem_size(), 0);
    return ElementRef{size_++};
  }
  int card_ = 0;
  int size_ = 0;
  std::vector<Set *> endpoint_sets_;
  std::vector<int32_t> endpoints_;
  std::vector<FieldData> fields_;
  std::string spatial_;
};

template <typename T, int... dims> T *FieldRef<T, dims...>::ptr(ElementRef e) const {
  FieldData &f = set_->field_at(idx_);
  return reinterpret_cast<T *>(f.data.data()) + (size_t)e.ident * kComps;
}

}  // namespace simit_gb300

#include "reorder.h"
#include "simit_function.h"
#include "map.h"
