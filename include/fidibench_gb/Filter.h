// Filter.h -- the reference's class Filter (cxx/Filter.h:25-230, cxx/Filter.cpp)
// rebuilt on the C-ABI of libfdb_upwind (include/fdb_filter.h), for one process
// and one GPU.
//
// Same constructor and public members as the reference, so its drivers
// (laplacian/cxx/laplacian.cxx, laplacian/cxx/testStencil2d.cxx) compile against
// this header once mpi.h is dropped:
//   Filter(globalDims, xmins, xmaxs, std::map<std::vector<int>, double> stencil)
//   void   setInData(double (*f)(const std::vector<double>&))          Filter.h:70
//   void   setInDataByIndices(double (*f)(const std::vector<size_t>&)) Filter.h:77
//   void   applyFilter()                                               Filter.h:84
//   void   copyOutToIn()                                               Filter.h:150
//   double computeCheckSum(const std::string& inOrOut)                 Filter.h:157
//   void   saveVTK(const std::string& filename)                        Filter.h:163
//   std::vector<double> getPosition(const std::vector<size_t>&)        Filter.h:58
//   std::vector<int> getSideFromOffset(const std::vector<int>&)        Filter.h:51
//   size_t getNumberOfGhostsFromOffset(const std::vector<int>&) const  Filter.h:99
//   int getRank() const (0), int getNumProcs() const (1), bool isDecompValid() const
//   void printInData(), void printOutData()
// The MPI-window members (fetch, getWindowIter, newWindow, deleteWindow,
// printSrcDataWindow, printDstDataWindow) have no one-process counterpart.
// Additions: setWrap(), iterate(), sync(), inData()/outData(), handle().
//
// Differences, by design: the data live on the GPU; errors throw
// std::runtime_error with fdb_last_error(); computeCheckSum is a fixed-order
// tree sum (the reference sums sequentially).  The neighbour wrap reproduces
// the reference's (see FDB_WRAP_REFERENCE) unless setWrap(FDB_WRAP_PERIODIC).
#ifndef FIDIBENCH_GB_FILTER_H
#define FIDIBENCH_GB_FILTER_H

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <numeric>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>
// (the standard headers the reference's Filter.h brings in through
// CubeDecomp.h, MultiArrayIter.h and writeVTK.h, so that drivers relying on
// them -- upwindMpi.cxx uses std::accumulate -- compile unchanged)

#include "../fdb_filter.h"
#include "../fdb_upwind.h"

namespace fdb {

inline void filter_check(int rc, const char* what) {
  if (rc != FDB_OK)
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) +
                             "): " + fdb_last_error());
}

class Filter {
 public:
  Filter(const std::vector<size_t>& globalDims, const std::vector<double>& xmins,
         const std::vector<double>& xmaxs, const std::map<std::vector<int>, double>& stencil)
      : globalDims_(globalDims), xmins_(xmins), xmaxs_(xmaxs), ndims_(globalDims.size()) {
    if (xmins.size() != ndims_ || xmaxs.size() != ndims_)
      throw std::invalid_argument("Filter: globalDims, xmins and xmaxs differ in length");
    std::vector<uint64_t> dims(globalDims.begin(), globalDims.end());
    std::vector<int> offs;
    std::vector<double> w;
    for (const auto& kv : stencil) {
      if (kv.first.size() != ndims_) throw std::invalid_argument("Filter: offset length");
      offs.insert(offs.end(), kv.first.begin(), kv.first.end());
      w.push_back(kv.second);
    }
    filter_check(fdb_filter_create((int)ndims_, dims.data(), xmins.data(), xmaxs.data(),
                                   (int)w.size(), offs.data(), w.data(), &h_),
                 "fdb_filter_create");
    ntot_ = 1;
    for (size_t n : globalDims) ntot_ *= n;
    // Filter.cpp:38-47 (rank 0 of one process; the decomposition is 1 x ... x 1)
    std::cout << "Number of procs: " << 1 << "\nglobal dimensions: ";
    for (size_t i = 0; i < ndims_; ++i) std::cout << globalDims[i] << ' ';
    std::cout << "\nDomain decomp ";
    for (size_t i = 0; i < ndims_; ++i) std::cout << 1 << ' ';
    std::cout << '\n';
  }
  ~Filter() { fdb_filter_destroy(h_); }
  Filter(const Filter&) = delete;
  Filter& operator=(const Filter&) = delete;

  std::vector<int> getSideFromOffset(const std::vector<int>& offset) {
    std::vector<int> side(ndims_, 0);
    for (size_t i = 0; i < ndims_; ++i)
      if (offset[i] != 0) side[i] = -offset[i] / std::abs(offset[i]);
    return side;
  }

  std::vector<double> getPosition(const std::vector<size_t>& globalInds) {
    std::vector<double> pos(ndims_);
    for (size_t i = 0; i < ndims_; ++i) {
      const double delta = (xmaxs_[i] - xmins_[i]) / double(globalDims_[i]);
      pos[i] = xmins_[i] + (globalInds[i] + 0.5) * delta;
    }
    return pos;
  }

  void setInData(double (*f)(const std::vector<double>&)) {
    std::vector<double> v(ntot_);
    std::vector<size_t> inds(ndims_);
    for (size_t i = 0; i < ntot_; ++i) {
      indices(i, inds);
      v[i] = f(getPosition(inds));
    }
    filter_check(fdb_filter_set_in_data(h_, v.data(), 0), "fdb_filter_set_in_data");
  }

  void setInDataByIndices(double (*f)(const std::vector<size_t>&)) {
    std::vector<double> v(ntot_);
    std::vector<size_t> inds(ndims_);
    for (size_t i = 0; i < ntot_; ++i) {
      indices(i, inds);
      v[i] = f(inds);
    }
    filter_check(fdb_filter_set_in_data(h_, v.data(), 0), "fdb_filter_set_in_data");
  }

  void applyFilter() { filter_check(fdb_filter_apply(h_), "fdb_filter_apply"); }
  void copyOutToIn() { filter_check(fdb_filter_copy_out_to_in(h_), "fdb_filter_copy_out_to_in"); }

  int getRank() const { return 0; }
  int getNumProcs() const { return 1; }
  bool isDecompValid() const { return true; }

  size_t getNumberOfGhostsFromOffset(const std::vector<int>& offset) const {
    size_t g = 0;
    for (int o : offset) g = (size_t)std::abs(o) > g ? (size_t)std::abs(o) : g;
    return g;
  }

  double computeCheckSum(const std::string& inOrOut) {
    double s = 0.0;
    filter_check(fdb_filter_checksum(h_, inOrOut == "input" ? 0 : 1, &s), "fdb_filter_checksum");
    return s;
  }

  // Filter.cpp:405-438 (stderr, rank 0)
  void printInData() { printData(0, "inData"); }
  void printOutData() { printData(1, "outData"); }

  // cxx/writeVTK.cpp:11-95 with the output data (Filter.cpp:487-535)
  void saveVTK(const std::string& filename) {
    if (ndims_ > 3) {
      std::cerr << "WARNING: writeVTK does not support more than 3 dimensions\n";
      return;
    }
    const std::vector<double> field = outData();
    double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {1.0, 1.0, 1.0};
    size_t cells[3] = {1, 1, 1};
    for (size_t d = 0; d < ndims_; ++d) {
      lo[d] = xmins_[d];
      hi[d] = xmaxs_[d];
      cells[d] = globalDims_[d];
    }
    const size_t nodes[3] = {cells[0] + 1, cells[1] + 1, cells[2] + 1};
    std::ofstream file(filename.c_str());
    file << "# vtk DataFile Version 2.0\n";
    file << "produced by laplacian\n";
    file << "ASCII\n";
    file << "DATASET STRUCTURED_GRID\n";
    file << "DIMENSIONS " << nodes[0] << ' ' << nodes[1] << ' ' << nodes[2] << '\n';
    file << "POINTS " << nodes[0] * nodes[1] * nodes[2] << " float\n";
    for (size_t k = 0; k < nodes[2]; ++k)
      for (size_t j = 0; j < nodes[1]; ++j)
        for (size_t i = 0; i < nodes[0]; ++i) {
          const double x = lo[0] + (hi[0] - lo[0]) * i / double(cells[0]);
          const double y = lo[1] + (hi[1] - lo[1]) * j / double(cells[1]);
          const double z = lo[2] + (hi[2] - lo[2]) * k / double(cells[2]);
          file << x << ' ' << y << ' ' << z << '\n';
        }
    file << "CELL_DATA " << cells[0] * cells[1] * cells[2] << '\n';
    file << "SCALARS " << "outData" << " float\n";
    file << "LOOKUP_TABLE default\n";
    for (double v : field) file << v << '\n';
  }

  // -- additions ------------------------------------------------------------
  void setWrap(int mode) { filter_check(fdb_filter_set_wrap(h_, mode), "fdb_filter_set_wrap"); }
  void iterate(int n) { filter_check(fdb_filter_iterate(h_, n), "fdb_filter_iterate"); }
  void sync() { filter_check(fdb_filter_synchronize(h_), "fdb_filter_synchronize"); }
  std::vector<double> inData() { return get(0); }
  std::vector<double> outData() { return get(1); }
  fdb_filter* handle() { return h_; }

 private:
  void indices(size_t bi, std::vector<size_t>& inds) const {
    size_t prod = 1;  // column-major (MultiArrayIter rowMajor = false)
    for (size_t d = 0; d < ndims_; ++d) {
      inds[d] = bi / prod % globalDims_[d];
      prod *= globalDims_[d];
    }
  }
  std::vector<double> get(int which) {
    std::vector<double> v(ntot_);
    filter_check(fdb_filter_get_data(h_, which, v.data(), 0), "fdb_filter_get_data");
    return v;
  }
  void printData(int which, const char* label) {
    const std::vector<double> v = get(which);
    std::vector<size_t> inds(ndims_);
    std::cerr << "[" << 0 << "] " << label << ": \n";
    for (size_t i = 0; i < ntot_; ++i) {
      indices(i, inds);
      std::cerr << "\t[" << 0 << "] inds = ";
      for (size_t j = 0; j < ndims_; ++j) std::cerr << inds[j] << ' ';
      std::cerr << " " << label << " = " << v[i] << '\n';
    }
  }

  std::vector<size_t> globalDims_;
  std::vector<double> xmins_, xmaxs_;
  size_t ndims_ = 0;
  size_t ntot_ = 0;
  fdb_filter* h_ = nullptr;
};

}  // namespace fdb

#ifndef FDB_NO_GLOBAL_FILTER
using fdb::Filter;
#endif

#endif  // FIDIBENCH_GB_FILTER_H
