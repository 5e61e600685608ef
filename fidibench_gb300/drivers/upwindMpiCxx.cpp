// upwindMpiCxx -- the reference's distributed upwind driver
// (upwind/cxx/upwindMpi.cxx:30-165) on the GB300 library for one process and
// one GPU, through the Filter facade include/fidibench_gb/Filter.h: the same
// stencil (the upwind step written as a Filter: centre 1 - sum_j s_j dt v_j /
// dx_j, and s_j dt v_j / dx_j at offset -s_j on axis j, s_j = sign v_j), the
// same corner initial condition set by indices, and the same output lines
// (per-step input/output check sums, times, "Check sum:").  The multi-GPU
// form of this run is fidibench_gb300.distributed.DistributedUpwind.
//   -numCells <int> (128)  -numSteps <int> (10)  -vtk  -h
#include <chrono>
#include <cstdlib>
#include <iostream>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "fidibench_gb/Filter.h"
#include "options.h"

namespace {

// 1 in the cell whose indices sum to zero (the corner), else 0
double corner(const std::vector<size_t>& inds) {
  size_t s = 0;
  for (size_t i : inds) s += i;
  return s == 0 ? 1.0 : 0.0;
}

}  // namespace

int main(int argc, char** argv) {
  fdb_drivers::Options o;
  o.values["-numCells"] = "128";
  o.help["-numCells"] = "Number of cells along each axis";
  o.values["-numSteps"] = "10";
  o.help["-numSteps"] = "Number of time steps";
  o.flags["-vtk"] = false;
  o.help["-vtk"] = "Write output to VTK file";
  o.flags["-h"] = false;
  o.help["-h"] = "Print help.";
  const bool success = fdb_drivers::parse(o, argc, argv);
  if (!success || o.flags["-h"]) {
    if (!success) std::cerr << "ERROR when parsing command line arguments\n";
    fdb_drivers::print_help(o, "Purpose: benchmark finite difference operations.", argv[0]);
    return 0;
  }
  const size_t numDims = 3;
  const size_t numCells = (size_t)std::atoi(o.values["-numCells"].c_str());
  const size_t numSteps = (size_t)std::atoi(o.values["-numSteps"].c_str());

  const std::vector<double> v(numDims, 1.0), lengths(numDims, 1.0);
  const double courant = 0.1;
  std::vector<double> dx(numDims);
  std::vector<int> sign(numDims);
  double dt = std::numeric_limits<double>::max();
  for (size_t j = 0; j < numDims; ++j) {
    dx[j] = lengths[j] / (double)numCells;
    const double val = courant * dx[j] / v[j];
    if (val < dt) dt = val;
    sign[j] = v[j] > 0 ? 1 : -1;
  }
  // the step as a stencil (upwindMpi.cxx:74-92): every weight rounded as there
  std::map<std::vector<int>, double> stencil;
  std::vector<int> offset(numDims, 0);
  double centre = 1.0;
  for (size_t j = 0; j < numDims; ++j) centre -= sign[j] * dt * v[j] / dx[j];
  stencil.insert(std::make_pair(offset, centre));
  for (size_t j = 0; j < numDims; ++j) {
    offset[j] = -sign[j];
    stencil.insert(std::make_pair(offset, sign[j] * dt * v[j] / dx[j]));
    offset[j] = 0;
  }
  try {
    Filter fltr(std::vector<size_t>(numDims, numCells), std::vector<double>(numDims, 0.0),
                lengths, stencil);
    const auto t0 = std::chrono::steady_clock::now();
    fltr.setInDataByIndices(corner);
    for (size_t i = 0; i < numSteps; ++i) {
      fltr.applyFilter();
      const double inSum = fltr.computeCheckSum("input");
      const double outSum = fltr.computeCheckSum("output");
      std::cout << "iter " << i << " check sum  in/out = " << inSum << " / " << outSum << '\n';
      fltr.copyOutToIn();
    }
    fltr.sync();
    const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (o.flags["-vtk"]) {
      std::cout << "Data will be written to file upMpi.vtk\n";
      fltr.saveVTK("upMpi.vtk");
    }
    const double outSum = fltr.computeCheckSum("output");
    std::cout << " times min/max/avg: " << t << '/' << t << '/' << t << " [seconds]\n";
    std::cout << "Check sum: " << outSum << '\n';
  } catch (const std::exception& e) {
    std::cerr << "ERROR: " << e.what() << '\n';
    return 1;
  }
  return 0;
}
