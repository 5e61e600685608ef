// testStencil2d -- the reference's general-stencil test driver
// (laplacian/cxx/testStencil2d.cxx) on the GB300 library, through the Filter
// facade include/fidibench_gb/Filter.h (one process, one GPU): the 2-D stencil
// {(0,0): 0, (1,0): 1, (0,-1): -1}, input 1 on every cell with a zero index,
// one applyFilter, the output printed by printOutData (stderr).
//   -numCells <int> (8)  -vtk  -h
#include <cstdlib>
#include <iostream>
#include <map>
#include <vector>

#include "fidibench_gb/Filter.h"
#include "options.h"

namespace {

double zero_index_cells(const std::vector<size_t>& inds) {
  size_t prod = 1;
  for (size_t i : inds) prod *= i;
  return prod == 0 ? 1.0 : 0.0;
}

}  // namespace

int main(int argc, char** argv) {
  fdb_drivers::Options o;
  o.values["-numCells"] = "8";
  o.help["-numCells"] = "Number of cells along each axis";
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
  const size_t n = (size_t)std::atoi(o.values["-numCells"].c_str());
  std::map<std::vector<int>, double> stencil;
  stencil.insert(std::make_pair(std::vector<int>{0, 0}, 0.0));
  stencil.insert(std::make_pair(std::vector<int>{1, 0}, 1.0));
  stencil.insert(std::make_pair(std::vector<int>{0, -1}, -1.0));
  try {
    Filter fltr(std::vector<size_t>(2, n), std::vector<double>(2, 0.0),
                std::vector<double>(2, 1.0), stencil);
    fltr.setInDataByIndices(zero_index_cells);
    fltr.applyFilter();
    fltr.printOutData();
    if (o.flags["-vtk"]) {
      std::cout << "Data will be written to file stencil2d.vtk\n";
      fltr.saveVTK("stencil2d.vtk");
    }
  } catch (const std::exception& e) {
    std::cerr << "ERROR: " << e.what() << '\n';
    return 1;
  }
  return 0;
}
