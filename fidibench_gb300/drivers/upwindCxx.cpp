// upwindCxx -- the reference's benchmark driver (upwind/cxx/upwind.cxx:139-217)
// on the GB300 library, through the C++ facade include/fidibench_gb/Upwind.h.
//
// Command line and output follow the reference so that its ctest cases
// (upwind/cxx/CMakeLists.txt:54-91: `upwindCxx 32 10`, PASS_REGULAR_EXPRESSION
// "[Cc]heck sum:[ ]*[1|0\.999]") run unchanged:
//   -numCells <int> (128)  -numSteps <int> (10)  -vtk  -std  -h
// Flags without a value toggle; tokens that are not options (such as the
// positional "32 10" of the ctest cases) are ignored; an unknown -option prints
// "<arg> is not a valid option." and the help text.  Added options:
//   -arith <auto|exact|fma|fixed>  -courant <double> (0.1)  -json
//   -velocity <vx,vy,vz> (1,1,1)  -adjoint (dL/dv of 0.5 sum f_T^2, and |dL/df0|)
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "fidibench_gb/Upwind.h"
#include "options.h"

namespace {

using fdb_drivers::Options;
using fdb_drivers::parse;

int arith_code(const std::string& s) {
  if (s == "exact") return FDB_ARITH_EXACT;
  if (s == "fma") return FDB_ARITH_FMA;
  if (s == "fixed") return FDB_ARITH_FIXED;
  return FDB_ARITH_AUTO;
}

}  // namespace

int main(int argc, char** argv) {
  const int ndims = 3;
  Options o;
  o.values["-numCells"] = "128";
  o.help["-numCells"] = "Number of cells along each axis";
  o.values["-numSteps"] = "10";
  o.help["-numSteps"] = "Number of time steps";
  o.values["-arith"] = "auto";
  o.help["-arith"] = "Step arithmetic: auto, exact, fma or fixed";
  o.values["-courant"] = "0.1";
  o.help["-courant"] = "Courant number used to pick dt";
  o.values["-velocity"] = "1,1,1";
  o.help["-velocity"] = "Velocity components vx,vy,vz (the reference driver's is 1,1,1)";
  o.flags["-adjoint"] = false;
  o.help["-adjoint"] = "Also print dL/dv of L = 0.5 sum f_T^2 (the adjoint)";
  o.flags["-vtk"] = false;
  o.help["-vtk"] = "Write output to VTK file";
  o.flags["-std"] = false;
  o.help["-std"] = "Print out spread of solution";
  o.flags["-json"] = false;
  o.help["-json"] = "Print a JSON timing line";
  o.flags["-h"] = false;
  o.help["-h"] = "Print help.";

  const bool success = parse(o, argc, argv);
  if (!success || o.flags["-h"]) {
    if (!success) std::cerr << "ERROR when parsing command line arguments\n";
    fdb_drivers::print_help(o, "Purpose: benchmark finite difference operations (GB300 library).",
                            argv[0]);
    return 0;
  }
  const int numTimeSteps = std::atoi(o.values["-numSteps"].c_str());
  const int n = std::atoi(o.values["-numCells"].c_str());
  std::cout << "Running with CUDA enabled (" << fdb_version() << ")\n";

  std::vector<size_t> numCells(ndims, (size_t)n);
  std::cout << "number of cells: ";
  for (size_t i = 0; i < numCells.size(); ++i) std::cout << ' ' << numCells[i];
  std::cout << '\n';
  std::cout << "number of time steps: " << numTimeSteps << '\n';

  std::vector<double> velocity(numCells.size(), 1.0);
  {
    std::stringstream vs(o.values["-velocity"]);
    std::string item;
    for (size_t j = 0; j < velocity.size() && std::getline(vs, item, ','); ++j)
      velocity[j] = std::atof(item.c_str());
  }
  std::vector<double> lengths(numCells.size(), 1.0);
  const double courant = std::atof(o.values["-courant"].c_str());
  double dt = std::numeric_limits<double>::max();
  for (size_t j = 0; j < velocity.size(); ++j) {
    const double dx = lengths[j] / numCells[j];
    if (velocity[j] == 0.0) continue;
    const double val = courant * dx / std::fabs(velocity[j]);
    dt = (val < dt ? val : dt);
  }

  try {
    Upwind<ndims> up(velocity, lengths, numCells);
    up.setArith(arith_code(o.values["-arith"]));
    if (o.flags["-vtk"]) up.saveVTK("up0.vtk");
    const std::vector<double> f0 = o.flags["-adjoint"] ? up.getField() : std::vector<double>();
    const auto t0 = std::chrono::steady_clock::now();
    up.advect(numTimeSteps, dt);
    const double cs = up.checksum();
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::cout << "check sum: " << cs << '\n';
    if (o.flags["-std"]) std::cout << "std      : " << up.std() << '\n';
    if (o.flags["-vtk"]) up.saveVTK("up1.vtk");
    if (o.flags["-adjoint"]) {
      // L = 0.5 sum f_T^2: lambda_T = f_T, then from f0 again
      const std::vector<double> lamT = up.getField();
      up.setInitialCondition(f0);
      std::vector<double> gv;
      const std::vector<double> g0 = up.adjoint(numTimeSteps, dt, lamT, &gv);
      double nrm = 0.0;
      for (double x : g0) nrm += x * x;
      std::cout << std::setprecision(17) << "dL/dv:";
      for (double x : gv) std::cout << ' ' << x;
      std::cout << "\n|dL/df0|: " << std::sqrt(nrm) << '\n' << std::setprecision(6);
    }
    if (o.flags["-json"]) {
      const double cells = (double)n * n * n;
      std::cout << "{\"cells\": " << cells << ", \"steps\": " << numTimeSteps
                << ", \"seconds\": " << sec << ", \"gcups\": " << cells * numTimeSteps / sec / 1e9
                << "}\n";
    }
  } catch (const std::exception& e) {
    std::cerr << "ERROR: " << e.what() << '\n';
    return 1;
  }
  return 0;
}
