// acc_driver.h -- the command line and output of the reference's OpenACC
// drivers (upwind/cxx/upwindAcc.cxx:117-172, upwindAcc2.cxx:137-193) on the
// GB300 library, through the C++ facade's std::vector<int> constructor (so
// the coefficients are rounded as those variants round them).  Included by
// upwindAccCxx.cpp (one advect(dt) call per step) and upwindAcc2Cxx.cpp (one
// advect(numSteps, dt) call, plus -std).
//
//   -numCells <int> (128)  -numSteps <int> (10)  -vtk  [-std: Acc2 only]  -h
// Added: -arith <auto|exact|fma|fixed>.  The ctest cases
// (upwind/cxx/CMakeLists.txt:93-107: `upwindAccCxx 32 10`,
// `upwindAcc2Cxx 32 10`, PASS_REGULAR_EXPRESSION "[Cc]heck sum:[ ]*[1|0\.999]")
// run unchanged: the positional tokens are not options and are ignored.
#ifndef FDB_DRIVERS_ACC_DRIVER_H
#define FDB_DRIVERS_ACC_DRIVER_H

#include <cstdlib>
#include <iostream>
#include <limits>
#include <string>
#include <vector>

#include "fidibench_gb/Upwind.h"
#include "options.h"

namespace fdb_drivers {

inline int acc_arith_code(const std::string& s) {
  if (s == "exact") return FDB_ARITH_EXACT;
  if (s == "fma") return FDB_ARITH_FMA;
  if (s == "fixed") return FDB_ARITH_FIXED;
  return FDB_ARITH_AUTO;
}

// one_step_calls: true = upwindAcc (advect(dt) per step), false = upwindAcc2
// (advect(numSteps, dt) and the -std option).
inline int run_acc_driver(int argc, char** argv, bool one_step_calls) {
  const int ndims = 3;
  Options o;
  o.values["-numCells"] = "128";
  o.help["-numCells"] = "Number of cells along each axis";
  o.values["-numSteps"] = "10";
  o.help["-numSteps"] = "Number of time steps";
  o.values["-arith"] = "auto";
  o.help["-arith"] = "Step arithmetic: auto, exact, fma or fixed";
  o.flags["-vtk"] = false;
  o.help["-vtk"] = "Write output to VTK file";
  if (!one_step_calls) {
    o.flags["-std"] = false;
    o.help["-std"] = "Print out spread of solution";
  }
  o.flags["-h"] = false;
  o.help["-h"] = "Print help.";

  const bool success = parse(o, argc, argv);
  if (!success) {
    std::cerr << "ERROR: wrong command line arguments\n";
    print_help(o, "Purpose: benchmark finite difference operations.", argv[0]);
    return 1;
  }
  if (o.flags["-h"]) {
    print_help(o, "Purpose: benchmark finite difference operations.", argv[0]);
    return 0;
  }
  const int n = std::atoi(o.values["-numCells"].c_str());
  const int numTimeSteps = std::atoi(o.values["-numSteps"].c_str());

  std::vector<int> numCells(ndims, n);
  std::cout << "number of cells: ";
  for (int c : numCells) std::cout << ' ' << c;
  std::cout << '\n';
  std::cout << "number of time steps: " << numTimeSteps << '\n';

  const std::vector<double> velocity(ndims, 1.0), lengths(ndims, 1.0);
  const double courant = 0.1;
  double dt = std::numeric_limits<double>::max();
  for (int j = 0; j < ndims; ++j) {
    const double val = courant * (lengths[j] / numCells[j]) / velocity[j];
    if (val < dt) dt = val;
  }
  try {
    fdb::Upwind<ndims> up(velocity, lengths, numCells);
    up.setArith(acc_arith_code(o.values["-arith"]));
    if (one_step_calls) {
      for (int s = 0; s < numTimeSteps; ++s) up.advect(dt);
    } else {
      up.advect(numTimeSteps, dt);
    }
    std::cout << "check sum: " << up.checksum() << '\n';
    if (!one_step_calls && o.flags["-std"]) std::cout << "std      : " << up.std() << '\n';
    if (o.flags["-vtk"]) up.saveVTK("up.vtk");
  } catch (const std::exception& e) {
    std::cerr << "ERROR: " << e.what() << '\n';
    return 1;
  }
  return 0;
}

}  // namespace fdb_drivers

#endif  // FDB_DRIVERS_ACC_DRIVER_H
