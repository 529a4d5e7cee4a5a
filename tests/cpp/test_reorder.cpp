// Set reordering of the C++ facade (simit_gb300/cpp/reorder.h) against the
// reference's reorder tests, restated:
//   test/reorder-tests.cpp:177-291  (TEST(Program, reorderInt))
//   test/reorder-tests.cpp:293-404  (TEST(Program, reorderDouble))
// and the properties reorder() keeps: orderings that are permutations,
// elements sorted by their sorted endpoint tuples, fields that move with
// their elements, errors for orderings that are not permutations and for a
// vertex set without a spatial field.  Host only: no GPU call.
#include <algorithm>
#include <cstdio>

#include "simit_gb300/cpp/simit.h"

using namespace simit_gb300;

static int g_fail = 0;
#define CHECK(cond)                                                      \
  do {                                                                   \
    if (!(cond)) {                                                       \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond);         \
      ++g_fail;                                                          \
    }                                                                    \
  } while (0)

// Two copies of a 3-vertex, 2-edge graph with vector fields on vertices
// (3 and 4 components) and edges (5); the second is reordered by the
// vertex ordering {2, 0, 1} and the edge ordering {1, 0}.  Every value is
// then found at its element's new index, and not at its old one.
template <typename T> static void test_reorder_fields() {
  Set V0, V1;
  Set E0(V0, V0), E1(V1, V1);
  auto x0 = V0.addField<T, 3>("x");
  auto a0 = V0.addField<T, 4>("a");
  auto t0 = E0.addField<T, 5>("x");
  auto x1 = V1.addField<T, 3>("x");
  auto a1 = V1.addField<T, 4>("a");
  auto t1 = E1.addField<T, 5>("x");
  std::vector<ElementRef> r0, r1, e0, e1;
  for (int i = 0; i < 3; ++i) {
    r0.push_back(V0.add());
    r1.push_back(V1.add());
    for (int q = 0; q < 3; ++q) {
      x0.get(r0[i])(q) = T(i);
      x1.get(r1[i])(q) = T(i);
    }
    for (int q = 0; q < 4; ++q) {
      a0.get(r0[i])(q) = T(3 + i);
      a1.get(r1[i])(q) = T(3 + i);
    }
  }
  const int ends[2][2] = {{1, 2}, {0, 1}};
  const T val[2] = {T(20), T(10)};
  for (int k = 0; k < 2; ++k) {
    e0.push_back(E0.add(r0[ends[k][0]], r0[ends[k][1]]));
    e1.push_back(E1.add(r1[ends[k][0]], r1[ends[k][1]]));
    for (int q = 0; q < 5; ++q) {
      t0.get(e0[k])(q) = val[k];
      t1.get(e1[k])(q) = val[k];
    }
  }
  std::vector<int> vo{2, 0, 1};
  std::vector<int> eo{1, 0};
  reorderVertexSet(E1, V1, vo);
  reorderEdgeSet(E1, eo);
  for (int i = 0; i < 3; ++i) {
    for (int q = 0; q < 3; ++q) {
      CHECK(x1.get(r1[vo[i]])(q) == x0.get(r0[i])(q));
      CHECK(x1.get(r1[i])(q) != x0.get(r0[i])(q));
    }
    for (int q = 0; q < 4; ++q) {
      CHECK(a1.get(r1[vo[i]])(q) == a0.get(r0[i])(q));
      CHECK(a1.get(r1[i])(q) != a0.get(r0[i])(q));
    }
  }
  for (int k = 0; k < 2; ++k)
    for (int q = 0; q < 5; ++q) {
      CHECK(t1.get(e1[eo[k]])(q) == t0.get(e0[k])(q));
      CHECK(t1.get(e1[k])(q) != t0.get(e0[k])(q));
    }
  // the endpoints: edge k's, relabelled, at its new index
  const auto &ep = E1.endpoints();
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 2; ++j) CHECK(ep[eo[k] * 2 + j] == vo[ends[k][j]]);
}

// An edge ordering that is not its own inverse: fields stay with endpoints.
static void test_edge_ordering_keeps_fields_with_endpoints() {
  Set V;
  Set E(V, V);
  auto w = E.addField<int>("w");
  std::vector<ElementRef> r;
  for (int i = 0; i < 4; ++i) r.push_back(V.add());
  const int ends[3][2] = {{0, 1}, {1, 2}, {2, 3}};
  for (int k = 0; k < 3; ++k) {
    ElementRef e = E.add(r[ends[k][0]], r[ends[k][1]]);
    w.set(e, 100 * ends[k][0] + ends[k][1]);
  }
  std::vector<int> eo{2, 0, 1};
  reorderEdgeSet(E, eo);
  const auto &ep = E.endpoints();
  for (int k = 0; k < 3; ++k) {
    const int a = ep[2 * k], b = ep[2 * k + 1];
    CHECK(w.get(ElementRef{k}) == 100 * a + b);
  }
  CHECK(ep[2 * eo[0]] == 0 && ep[2 * eo[0] + 1] == 1);
}

static void test_errors() {
  Set V;
  Set E(V, V);
  V.addField<double, 3>("x");
  std::vector<ElementRef> r;
  for (int i = 0; i < 3; ++i) r.push_back(V.add());
  E.add(r[0], r[1]);
  int thrown = 0;
  try {
    std::vector<int> bad{0, 0, 1};
    reorderVertexSet(E, V, bad);
  } catch (const SimitException &) {
    ++thrown;
  }
  try {
    std::vector<int> shortv{0, 1};
    reorderVertexSet(E, V, shortv);
  } catch (const SimitException &) {
    ++thrown;
  }
  try {
    reorder(E, V);  // no spatial field
  } catch (const SimitException &) {
    ++thrown;
  }
  try {
    V.setSpatialField("no_such_field");
  } catch (const SimitException &) {
    ++thrown;
  }
  CHECK(thrown == 4);
  // nothing moved
  CHECK(E.endpoints()[0] == 0 && E.endpoints()[1] == 1);
}

// reorder() on a 4x4x4 point lattice with a tet-like 4-endpoint set: both
// orderings are permutations, the positions and element fields follow, and
// the elements come sorted by their sorted endpoint tuples.
static void test_reorder_lattice() {
  Set V;
  Set T(V, V, V, V);
  auto x = V.addField<double, 3>("x");
  auto id = V.addField<int>("id");
  auto tag = T.addField<int, 4>("tag");
  const int s = 4;
  std::vector<ElementRef> r;
  for (int i = 0; i < s; ++i)
    for (int j = 0; j < s; ++j)
      for (int k = 0; k < s; ++k) {
        r.push_back(V.add());
        x.set(r.back(), {0.25 * i, 0.5 * j, 1.0 * k});
        id.set(r.back(), (int)r.size() - 1);
      }
  auto vid = [&](int i, int j, int k) { return (i * s + j) * s + k; };
  std::vector<std::array<int, 4>> els;
  for (int i = 0; i + 1 < s; ++i)
    for (int j = 0; j + 1 < s; ++j)
      for (int k = s - 2; k >= 0; --k)
        els.push_back({vid(i + 1, j, k), vid(i, j + 1, k), vid(i, j, k + 1), vid(i, j, k)});
  for (auto &e : els) {
    ElementRef t = T.add(r[e[0]], r[e[1]], r[e[2]], r[e[3]]);
    tag.set(t, {e[0], e[1], e[2], e[3]});
  }
  const int n = (int)r.size(), nE = (int)els.size();
  std::vector<double> x0((size_t)n * 3);
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) x0[i * 3 + q] = x.get(r[i])(q);
  std::vector<int> eo, vo;
  V.setSpatialField("x");
  reorder(T, V, eo, vo);
  CHECK((int)vo.size() == n && (int)eo.size() == nE);
  std::vector<int> sv(vo), se(eo);
  std::sort(sv.begin(), sv.end());
  std::sort(se.begin(), se.end());
  for (int i = 0; i < n; ++i) CHECK(sv[i] == i);
  for (int i = 0; i < nE; ++i) CHECK(se[i] == i);
  bool moved = false;
  for (int i = 0; i < n; ++i) {
    moved = moved || vo[i] != i;
    CHECK(id.get(r[vo[i]]) == i);
    for (int q = 0; q < 3; ++q) CHECK(x.get(r[vo[i]])(q) == x0[i * 3 + q]);
  }
  CHECK(moved);
  const auto &ep = T.endpoints();
  std::array<int, 4> prev{-1, -1, -1, -1};
  for (int k = 0; k < nE; ++k) {
    std::array<int, 4> cur;
    for (int j = 0; j < 4; ++j) {
      // element k carries its old endpoints in `tag`: relabelled they are
      // its endpoints now
      CHECK(ep[k * 4 + j] == vo[tag.get(ElementRef{k})(j)]);
      cur[j] = ep[k * 4 + j];
    }
    std::sort(cur.begin(), cur.end());
    CHECK(!(cur < prev));
    prev = cur;
  }
}

int main() {
  try {
    test_reorder_fields<int>();
    test_reorder_fields<double>();
    test_edge_ordering_keeps_fields_with_endpoints();
    test_errors();
    test_reorder_lattice();
  } catch (const std::exception &e) {
    std::printf("FAIL exception: %s\n", e.what());
    return 2;
  }
  std::printf(g_fail ? "%d failures\n" : "all passed\n", g_fail);
  return g_fail ? 1 : 0;
}
