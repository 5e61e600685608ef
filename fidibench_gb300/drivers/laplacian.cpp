// laplacian -- the reference's Laplacian driver (laplacian/cxx/laplacian.cxx)
// on the GB300 library, through the C++ facade include/fidibench_gb/Filter.h
// (one process, one GPU: no MPI).
//
// Command line and output follow the reference, so its ctest cases
// (laplacian/cxx/CMakeLists.txt: `laplacian -numDims 2|3 -numCells N`,
// PASS_REGULAR_EXPRESSION "[Cc]heck sums:[ ]*") run unchanged:
//   -numCells <int> (8000)  -numDims <int> (2)  -vtk  -h
// The input is prod_i sin(2 pi x_i) at the cell centres of the unit cube, the
// stencil -2 numDims at the centre and +1 at +-1 along every axis, and the
// timed loop 10 x (applyFilter; copyOutToIn).  Added options:
//   -periodic (periodic wrap for every N, see FDB_WRAP_PERIODIC)  -json
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "fidibench_gb/Filter.h"
#include "options.h"

namespace {

double func(const std::vector<double>& pos) {
  double res = 1;
  for (size_t i = 0; i < pos.size(); ++i) res *= sin(2.0 * M_PI * pos[i]);
  return res;
}

}  // namespace

int main(int argc, char** argv) {
  fdb_drivers::Options o;
  o.values["-numCells"] = "8000";
  o.help["-numCells"] = "Number of cells along each axis";
  o.values["-numDims"] = "2";
  o.help["-numDims"] = "Number of dimensions";
  o.flags["-vtk"] = false;
  o.help["-vtk"] = "Write output to VTK file";
  o.flags["-periodic"] = false;
  o.help["-periodic"] = "Periodic neighbour wrap for every grid size";
  o.flags["-json"] = false;
  o.help["-json"] = "Print a JSON timing line";
  o.flags["-h"] = false;
  o.help["-h"] = "Print help.";

  const bool success = fdb_drivers::parse(o, argc, argv);
  if (!success || o.flags["-h"]) {
    if (!success) std::cerr << "ERROR when parsing command line arguments\n";
    fdb_drivers::print_help(o, "Purpose: benchmark finite difference operations.", argv[0]);
    return 0;
  }
  const size_t numCells = (size_t)std::atoi(o.values["-numCells"].c_str());
  const size_t numDims = (size_t)std::atoi(o.values["-numDims"].c_str());

  // the stencil (laplacian.cxx:57-66)
  std::map<std::vector<int>, double> stencil;
  std::vector<int> offset(numDims, 0);
  stencil.insert(std::pair<std::vector<int>, double>(offset, -2.0 * numDims));
  for (size_t i = 0; i < numDims; ++i) {
    offset[i] = 1;
    stencil.insert(std::pair<std::vector<int>, double>(offset, 1.0));
    offset[i] = -1;
    stencil.insert(std::pair<std::vector<int>, double>(offset, 1.0));
    offset[i] = 0;
  }
  std::vector<size_t> globalDims(numDims, numCells);
  std::vector<double> xmins(numDims, 0.0);
  std::vector<double> xmaxs(numDims, 1.0);

  try {
    Filter fltr(globalDims, xmins, xmaxs, stencil);
    if (o.flags["-periodic"]) fltr.setWrap(FDB_WRAP_PERIODIC);
    fltr.setInData(func);
    fltr.sync();
    const auto t0 = std::chrono::steady_clock::now();
    const size_t numIter = 10;
    for (size_t i = 0; i < numIter; ++i) {
      fltr.applyFilter();
      fltr.copyOutToIn();
    }
    fltr.sync();
    const double walltime =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (o.flags["-vtk"]) {
      std::cout << "Data will be written to file laplacian.vtk\n";
      fltr.saveVTK("laplacian.vtk");
    }
    const double inSum = fltr.computeCheckSum("input");
    const double outSum = fltr.computeCheckSum("output");
    std::cout << "Laplace times min/max/avg: " << walltime << '/' << walltime << '/' << walltime
              << " [seconds]\n";
    std::cout << "Check sums: input = " << inSum << " output = " << outSum << '\n';
    if (o.flags["-json"]) {
      double cells = 1.0;
      for (size_t n : globalDims) cells *= (double)n;
      std::cout << "{\"cells\": " << cells << ", \"iterations\": " << numIter
                << ", \"seconds\": " << walltime
                << ", \"gcups\": " << cells * numIter / walltime / 1e9 << "}\n";
    }
  } catch (const std::exception& e) {
    std::cerr << "ERROR: " << e.what() << '\n';
    return 1;
  }
  return 0;
}
