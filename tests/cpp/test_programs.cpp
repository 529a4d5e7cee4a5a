// The reference's program tests, written against the C++ facade
// (simit_gb300/cpp/simit.h) exactly as the reference writes them against
// simit::Set / simit::Function, with the reference's golden values:
//   test/program-isprings.cpp:91-175  (TEST(Program, isprings))
//   test/program-cg-test.cpp:10-44    (TEST(Program, cg))
//   test/program-fem-test.cpp:14-106  (TEST(Program, femTet), bar2k mesh)
//   test/reorder-tests.cpp:403-471    (reorderFemSpecificTest: the same run on
//                                      the Hilbert-reordered mesh; reorderFemTest,
//                                      reorderCube: reordered against original)
// Exit code 0 when every value is within 1e-13 (SIMIT_ASSERT_FLOAT_EQ).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>

#include "simit_gb300/cpp/simit.h"

using namespace simit_gb300;

static int g_fail = 0;
#define ASSERT_NEAR13(expected, actual)                                                   \
  do {                                                                                    \
    double e_ = (expected), a_ = (actual);                                                \
    if (!(std::fabs(e_ - a_) <= 1e-13)) {                                                 \
      std::printf("FAIL %s:%d expected %.17g got %.17g\n", __FILE__, __LINE__, e_, a_);   \
      ++g_fail;                                                                           \
    }                                                                                     \
  } while (0)

static void test_isprings() {
  double l0_ = 1.0, stiffness = 100.00, density = 1000.0, radius = 0.01, PI_ = 3.14159265358979;
  double zfloor = 0.4;
  Set points;
  auto x = points.addField<double, 3>("x");
  auto v = points.addField<double, 3>("v");
  auto m = points.addField<double>("m");
  auto fixed = points.addField<bool>("fixed");
  Set springs(points, points);
  auto k = springs.addField<double>("k");
  auto l0 = springs.addField<double>("l0");
  ElementRef p0 = points.add(), p1 = points.add(), p2 = points.add();
  x(p0) = {0.0, 0.0, 0.0};
  x(p1) = {0.0, 0.0, 1.0};
  x(p2) = {0.0, 0.0, 2.0};
  v(p0) = {0.0, 0.0, 0.0};
  v(p1) = {0.0, 0.0, 0.0};
  v(p2) = {0.0, 0.0, 0.0};
  for (ElementRef p : {p0, p1, p2}) m(p) = PI_ * radius * radius * l0_ * density;
  ElementRef s0 = springs.add(p0, p1), s1 = springs.add(p1, p2);
  l0(s0) = l0_;
  l0(s1) = l0_;
  k(s0) = stiffness;
  k(s1) = stiffness;
  for (ElementRef p : {p0, p1, p2}) fixed(p) = x(p)(2) < zfloor;
  Function func("isprings");
  func.bind("points", &points);
  func.bind("springs", &springs);
  for (int i = 0; i < 10; ++i) func.runSafe();
  ASSERT_NEAR13(0.0, v(p1)(0));
  ASSERT_NEAR13(-0.54482994491692449, v(p1)(2));
  ASSERT_NEAR13(-0.8480293605755741, v(p2)(2));
  ASSERT_NEAR13(0.96180188527075183, x(p1)(2));
  ASSERT_NEAR13(1.9500008677096612, x(p2)(2));
  ASSERT_NEAR13(0.0, x(p0)(2));
}

static void test_cg() {
  Set points;
  auto b = points.addField<double>("b");
  auto c = points.addField<double>("c");
  auto id = points.addField<int>("id");
  (void)id;
  ElementRef p0 = points.add(), p1 = points.add(), p2 = points.add();
  b.set(p0, 1.0);
  b.set(p1, 2.0);
  b.set(p2, 3.0);
  Set springs(points, points);
  auto a = springs.addField<double>("a");
  ElementRef s0 = springs.add(p0, p1), s1 = springs.add(p1, p2);
  a.set(s0, 4.0);
  a.set(s1, 5.0);
  Function func("cg");
  func.bind("points", &points);
  func.bind("springs", &springs);
  func.runSafe();
  ASSERT_NEAR13(0.95883777239709455653, (double)c.get(p0));
  ASSERT_NEAR13(1.98789346246973352983, (double)c.get(p1));
  ASSERT_NEAR13(3.05326876513317202466, (double)c.get(p2));
}

// TetGen .node/.ele reader (the fixture copies of test/input/program/fem/bar2k)
static bool load_tet(const std::string &prefix, std::vector<double> &xv,
                     std::vector<std::array<int, 4>> &ev) {
  std::ifstream nf(prefix + ".node"), ef(prefix + ".ele");
  if (!nf || !ef) return false;
  int nv, d0, d1, d2;
  nf >> nv >> d0 >> d1 >> d2;
  xv.resize((size_t)nv * 3);
  for (int i = 0; i < nv; ++i) {
    int idx;
    nf >> idx >> xv[i * 3] >> xv[i * 3 + 1] >> xv[i * 3 + 2];
  }
  int ne, per, attr;
  ef >> ne >> per >> attr;
  ev.resize(ne);
  for (int i = 0; i < ne; ++i) {
    int idx;
    ef >> idx >> ev[i][0] >> ev[i][1] >> ev[i][2] >> ev[i][3];
  }
  return true;
}

// femTet (test/program-fem-test.cpp:14-106's set-up) for 10 steps on the
// TetGen mesh `prefix`, optionally reordered first (test/reorder-tests.cpp:
// the femTest helper); the positions of the vertices by original index.
static std::vector<double> run_femtet(const std::string &prefix, bool reordered) {
  std::vector<double> xv;
  std::vector<std::array<int, 4>> ev;
  if (!load_tet(prefix, xv, ev)) {
    std::printf("FAIL cannot read %s\n", prefix.c_str());
    ++g_fail;
    return {};
  }
  Set verts;
  Set tets(verts, verts, verts, verts);
  auto x = verts.addField<double, 3>("x");
  auto v = verts.addField<double, 3>("v");
  auto fe = verts.addField<double, 3>("fe");
  auto c = verts.addField<int>("c");
  auto m = verts.addField<double>("m");
  auto u = tets.addField<double>("u");
  auto l = tets.addField<double>("l");
  auto W = tets.addField<double>("W");
  auto B = tets.addField<double, 3, 3>("B");
  (void)fe; (void)W; (void)B;
  double E = 5e3, nu = 0.45;
  double uval = 0.5 * E / nu, lval = E * nu / ((1 + nu) * (1 - 2 * nu));
  double eps = 0.0001;
  std::vector<ElementRef> refs;
  for (size_t i = 0; i < xv.size() / 3; ++i) {
    refs.push_back(verts.add());
    ElementRef p = refs.back();
    x.set(p, {xv[i * 3], xv[i * 3 + 1], xv[i * 3 + 2]});
    v.set(p, {0.1, 0.0, 0.1});
    c.set(p, 0);
    m.set(p, 0.0);
    if (xv[i * 3 + 1] < eps) {
      c.set(p, 1);
      v.set(p, {0, 0, 0});
    }
  }
  for (auto &e : ev) {
    ElementRef t = tets.add(refs[e[0]], refs[e[1]], refs[e[2]], refs[e[3]]);
    u.set(t, uval);
    l.set(t, lval);
  }
  // vertex i's values are at index at[i] after the optional reordering
  std::vector<int> at(refs.size());
  for (size_t i = 0; i < at.size(); ++i) at[i] = (int)i;
  if (reordered) {
    std::vector<int> edgeOrdering;
    verts.setSpatialField("x");
    reorder(tets, verts, edgeOrdering, at);
  }
  Function pre("femTet.init");
  pre.bind("verts", &verts);
  pre.bind("tets", &tets);
  pre.init();
  pre.runSafe();
  Function step("femTet");
  step.bind("verts", &verts);
  step.bind("tets", &tets);
  step.init();
  for (int i = 0; i < 10; ++i) step.runSafe();
  std::vector<double> out(xv.size());
  for (size_t i = 0; i < at.size(); ++i)
    for (int q = 0; q < 3; ++q) out[i * 3 + q] = x.get(refs[at[i]])(q);
  return out;
}

// TEST(Program, femTet) and, reordered, TEST(Program, reorderFemSpecificTest):
// the golden displacements of vertices 100, 200 and 300.
static void test_femtet(const std::string &golden_dir, bool reordered) {
  std::vector<double> x = run_femtet(golden_dir + "/bar2k", reordered);
  if (x.empty()) return;
  ASSERT_NEAR13(0.010771915616785779, x[100 * 3 + 0]);
  ASSERT_NEAR13(0.058853573999788439, x[100 * 3 + 1]);
  ASSERT_NEAR13(0.030899457015375883, x[100 * 3 + 2]);
  ASSERT_NEAR13(0.0028221631202928516, x[200 * 3 + 0]);
  ASSERT_NEAR13(0.017969982607667911, x[200 * 3 + 1]);
  ASSERT_NEAR13(0.012885386063393013, x[200 * 3 + 2]);
  ASSERT_NEAR13(0.02411959295647129, x[300 * 3 + 0]);
  ASSERT_NEAR13(0.052036155669135678, x[300 * 3 + 1]);
  ASSERT_NEAR13(0.030173075240629205, x[300 * 3 + 2]);
}

// TEST(Program, reorderFemTest) / reorderCube (test/reorder-tests.cpp:
// 453-471): every vertex of the reordered run within 1e-5 of the original
// run (SIMIT_ASSERT_FLOAT_NEAR_EQ).
static void test_reorder_invariance(const std::string &prefix) {
  std::vector<double> a = run_femtet(prefix, false), b = run_femtet(prefix, true);
  if (a.empty() || a.size() != b.size()) {
    std::printf("FAIL %s: runs of different sizes\n", prefix.c_str());
    ++g_fail;
    return;
  }
  double worst = 0;
  for (size_t i = 0; i < a.size(); ++i) worst = std::max(worst, std::fabs(a[i] - b[i]));
  if (!(worst <= 1e-5)) {
    std::printf("FAIL %s: reordered run differs by %.3g\n", prefix.c_str(), worst);
    ++g_fail;
  }
  std::printf("reorder %s: max |x_reordered - x| = %.3g\n", prefix.c_str(), worst);
}

static void test_bind_errors() {
  Set points;
  Function f("isprings");
  bool threw = false;
  try {
    f.bind("no_such_set", &points);
  } catch (const SimitException &) {
    threw = true;
  }
  if (!threw) {
    std::printf("FAIL bind of an unknown name did not throw\n");
    ++g_fail;
  }
}

int main(int argc, char **argv) {
  const std::string golden = argc > 1 ? argv[1] : "tests/golden";
  try {
    test_isprings();
    test_cg();
    test_femtet(golden, false);
    test_femtet(golden, true);
    test_reorder_invariance(golden + "/bar2k");
    test_reorder_invariance(golden + "/cube");
    test_bind_errors();
  } catch (const std::exception &e) {
    std::printf("FAIL exception: %s\n", e.what());
    return 2;
  }
  std::printf(g_fail ? "%d failures\n" : "all passed\n", g_fail);
  return g_fail ? 1 : 0;
}
