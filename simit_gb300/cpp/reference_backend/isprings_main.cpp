// The reference's isprings program test (test/program-isprings.cpp:91-175)
// run through the reference's own simit::Program and simit::Function with
// the GB300 backend: the same three-vertex chain, ten runSafe calls, then
// v and x printed with 17 significant digits, one "name value" per line.
// When no GPU is present the backend stops at the device (sg_ctx_create);
// the driver then prints the backend's view of the bound sets and the
// error, and exits 0 -- the run got through the reference's frontend,
// lowering, backend factory and Function binding to the C ABI.
//
// Usage: isprings_main <path of the reference's isprings.sim>
//        isprings_main --compile <program.sim> <function>
//          (compile only: prints "compiled: ..." or "refused", the backend's
//          message on stderr)
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>

#include "error.h"
#include "graph.h"
#include "init.h"
#include "program.h"

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s isprings.sim\n", argv[0]);
    return 2;
  }
  simit::init("cpu", 8);
  if (std::string(argv[1]) == "--compile" && argc >= 4) {
    simit::Program program;
    if (program.loadFile(argv[2]) != 0) {
      std::cout << "load failed: " << program.getDiagnostics().getMessage() << std::endl;
      return 3;
    }
    try {
      simit::Function f = program.compile(argv[3]);
      std::cout << "compiled: " << f << std::endl;
    } catch (const simit::SimitException &) {
      std::cout << "refused" << std::endl;
    }
    return 0;
  }

  const double l0_ = 1.0, stiffness = 100.0, density = 1000.0, radius = 0.01;
  const double pi = 3.14159265358979, zfloor = 0.4;

  simit::Set points;
  simit::FieldRef<double, 3> x = points.addField<double, 3>("x");
  simit::FieldRef<double, 3> v = points.addField<double, 3>("v");
  simit::FieldRef<double> m = points.addField<double>("m");
  simit::FieldRef<bool> fixed = points.addField<bool>("fixed");
  simit::Set springs(points, points);
  simit::FieldRef<double> k = springs.addField<double>("k");
  simit::FieldRef<double> l0 = springs.addField<double>("l0");

  simit::ElementRef p[3];
  for (int i = 0; i < 3; ++i) {
    p[i] = points.add();
    x(p[i]) = {0.0, 0.0, (double)i};
    v(p[i]) = {0.0, 0.0, 0.0};
    m(p[i]) = pi * radius * radius * l0_ * density;
  }
  for (int i = 0; i < 2; ++i) {
    simit::ElementRef s = springs.add(p[i], p[i + 1]);
    l0(s) = l0_;
    k(s) = stiffness;
  }
  for (int i = 0; i < 3; ++i) fixed(p[i]) = x(p[i])(2) < zfloor;

  simit::Program program;
  if (program.loadFile(argv[1]) != 0) {
    std::cout << "load failed: " << program.getDiagnostics().getMessage() << std::endl;
    return 3;
  }
  simit::Function func = program.compile("main");
  if (!func.defined()) {
    std::cout << "compile failed" << std::endl;
    return 4;
  }
  func.bind("points", &points);
  func.bind("springs", &springs);
  std::cout << "compiled: " << func << std::endl;
  try {
    for (int i = 0; i < 10; ++i) func.runSafe();
  } catch (const simit::SimitException &) {
    std::cout << "stopped: " << func << std::endl;
    std::cout << "device unavailable" << std::endl;
    return 0;
  }
  char buf[64];
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) {
      std::snprintf(buf, sizeof buf, "v(p%d)(%d) %.17g", i, c, (double)v(p[i])(c));
      std::cout << buf << "\n";
    }
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) {
      std::snprintf(buf, sizeof buf, "x(p%d)(%d) %.17g", i, c, (double)x(p[i])(c));
      std::cout << buf << "\n";
    }
  std::cout << "ran 10 steps" << std::endl;
  return 0;
}
