// Upwind.h -- the reference's C++ class Upwind<NDIMS> (upwind/cxx/upwind.cxx:19-135)
// rebuilt on the C-ABI of libfdb_upwind (include/fdb_upwind.h).
//
// Same constructor and member signatures as the reference, so a driver written
// against upwind.cxx (or its OpenACC variants) compiles against this header
// unchanged:
//   Upwind(const std::vector<double>& velocity, const std::vector<double>& lengths,
//          const std::vector<size_t>& numCells)                 upwind.cxx:23-49
//   Upwind(const std::vector<double>& velocity, const std::vector<double>& lengths,
//          const std::vector<int>& numCells)                    upwindAcc.cxx:17-47,
//                                                               upwindAcc2.cxx:18-50
//   void   advect(int numTimeSteps, double deltaTime)           upwind.cxx:51-86,
//                                                               upwindAcc2.cxx:52-99
//   void   advect(double deltaTime)      (one step)             upwindAcc.cxx:49-90
//   void   saveVTK(const std::string& filename)                 saveVTK.h:1-60
//   double checksum() const                                     upwind.cxx:91-93
//   double std() const                                          upwind.cxx:95-103
//   void   print() const                                        upwind.cxx:105-109
// Additions: setInitialCondition(), getField(), setArith(), handle(),
// adjoint(), advectTransposed(), advectHostStream().
//
// Differences, by design: the field lives on the GPU (copied to the host only
// by print/saveVTK/getField); errors throw std::runtime_error carrying
// fdb_last_error() (the reference has no error reporting); advect() returns
// once the work is enqueued and the next host-visible call synchronises.
#ifndef FIDIBENCH_GB_UPWIND_H
#define FIDIBENCH_GB_UPWIND_H

#include <cstddef>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../fdb_upwind.h"

namespace fdb {

inline void check(int rc, const char* what) {
  if (rc != FDB_OK)
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) +
                             "): " + fdb_last_error());
}

template <size_t NDIMS>
class Upwind {
 public:
  Upwind(const std::vector<double>& velocity, const std::vector<double>& lengths,
         const std::vector<size_t>& numCells)
      : v_(velocity), lengths_(lengths), numCells_(numCells) {
    create();
  }

  // The OpenACC variants' constructor.  They precompute v_j * up_j / dx_j and
  // multiply by deltaTime in each update (upwindAcc.cxx:45,79), a coefficient
  // rounding that differs from upwind.cxx:72 in the last bit; the handle is
  // set to that form (FDB_COEFF_PRODUCT), so FDB_ARITH_EXACT reproduces these
  // variants bit for bit.
  Upwind(const std::vector<double>& velocity, const std::vector<double>& lengths,
         const std::vector<int>& numCells)
      : v_(velocity), lengths_(lengths) {
    for (int n : numCells) {
      if (n <= 0) throw std::invalid_argument("Upwind: numCells must be positive");
      numCells_.push_back((size_t)n);
    }
    create();
    check(fdb_upwind_set_coeff_form(h_, FDB_COEFF_PRODUCT), "fdb_upwind_set_coeff_form");
  }
  ~Upwind() { fdb_upwind_destroy(h_); }
  Upwind(const Upwind&) = delete;
  Upwind& operator=(const Upwind&) = delete;

  void advect(int numTimeSteps, double deltaTime) {
    check(fdb_upwind_advect(h_, numTimeSteps, deltaTime), "fdb_upwind_advect");
  }

  // One time step (upwindAcc.cxx:49-90).
  void advect(double deltaTime) { advect(1, deltaTime); }

  double checksum() const {
    double s = 0.0;
    check(fdb_upwind_checksum(h_, &s), "fdb_upwind_checksum");
    return s;
  }

  double std() const {
    double s = 0.0;
    check(fdb_upwind_std(h_, &s), "fdb_upwind_std");
    return s;
  }

  void print() const {
    std::vector<double> f = getField();
    for (size_t i = 0; i < f.size(); ++i) std::cout << i << " " << f[i] << '\n';
  }

  // ASCII RECTILINEAR_GRID, the reference writer's layout (saveVTK.h:1-60).
  void saveVTK(const std::string& filename) {
    std::vector<double> f = getField();
    std::fstream file;
    file.open(filename.c_str(), std::ios_base::out);
    file << "# vtk DataFile Version 2.0\nupwind.cxx\nASCII\nDATASET RECTILINEAR_GRID\n";
    file << "DIMENSIONS";
    file << ' ' << (NDIMS > 2 ? numCells_[NDIMS > 2 ? 2 : 0] + 1 : 1);
    file << ' ' << (NDIMS > 1 ? numCells_[NDIMS > 1 ? 1 : 0] + 1 : 1);
    file << ' ' << numCells_[0] + 1;
    axis(file, "X_COORDINATES", NDIMS > 2 ? 2 : -1);
    axis(file, "Y_COORDINATES", NDIMS > 1 ? 1 : -1);
    axis(file, "Z_COORDINATES", 0);
    file << "\nCELL_DATA " << ntot_ << '\n';
    file << "SCALARS f double 1\nLOOKUP_TABLE default\n";
    for (size_t i = 0; i < ntot_; ++i) {
      file << f[i] << " ";
      if ((i + 1) % 10 == 0) file << '\n';
    }
    file << '\n';
  }

  // setInitialCondition: replaces the constructor's f = 0, f[0] = 1.
  void setInitialCondition(const std::vector<double>& f) {
    if (f.size() != ntot_) throw std::invalid_argument("setInitialCondition: wrong size");
    check(fdb_upwind_set_field(h_, f.data(), 0), "fdb_upwind_set_field");
  }

  std::vector<double> getField() const {
    std::vector<double> f(ntot_);
    check(fdb_upwind_get_field(h_, f.data(), 0), "fdb_upwind_get_field");
    return f;
  }

  // Gradients of a loss L(f_T) given lambdaT = dL/df_T (no reference
  // counterpart; fdb_upwind_adjoint): runs advect(numTimeSteps, deltaTime)
  // from the current field with a checkpoint every checkpointEvery steps
  // (0: about sqrt(numTimeSteps)), then the transposed steps.  Returns
  // dL/df0; gradVelocity (nullable) receives dL/dv (NDIMS values).  Without
  // gradVelocity only dL/df0 is computed (the transposed problem alone, no
  // checkpoints).  The field ends at f_T, as after advect.
  std::vector<double> adjoint(int numTimeSteps, double deltaTime,
                              const std::vector<double>& lambdaT,
                              std::vector<double>* gradVelocity = nullptr,
                              int checkpointEvery = 0) {
    if (lambdaT.size() != ntot_) throw std::invalid_argument("adjoint: wrong lambdaT size");
    std::vector<double> g(ntot_);
    std::vector<double> gv(NDIMS, 0.0);
    check(fdb_upwind_adjoint(h_, numTimeSteps, deltaTime, lambdaT.data(), g.data(),
                             gradVelocity ? gv.data() : nullptr, checkpointEvery, 0),
          "fdb_upwind_adjoint");
    if (gradVelocity) *gradVelocity = gv;
    return g;
  }

  // The transpose of advect alone (fdb_upwind_advect_transposed): returns
  // (A^T)^numTimeSteps lambda -- dL/df0 for a caller that already holds f_T
  // -- without touching the field.
  std::vector<double> advectTransposed(int numTimeSteps, double deltaTime,
                                       const std::vector<double>& lambda) {
    if (lambda.size() != ntot_) throw std::invalid_argument("advectTransposed: wrong size");
    std::vector<double> out(ntot_);
    check(fdb_upwind_advect_transposed(h_, numTimeSteps, deltaTime, lambda.data(), out.data(), 0),
          "fdb_upwind_advect_transposed");
    return out;
  }

  // The driver's cycle (set the field, advect, checksum) over many host
  // fields (fdb_upwind_advect_host_stream): fields[k] (size() doubles each)
  // is advected in place and its checksum returned; the next upload and the
  // previous download overlap each advect when the buffers are pinned.  The
  // handle's field ends at the last result.
  std::vector<double> advectHostStream(const std::vector<double*>& fields, int numTimeSteps,
                                       double deltaTime) {
    std::vector<double> sums(fields.size());
    std::vector<const double*> in(fields.begin(), fields.end());
    check(fdb_upwind_advect_host_stream(h_, (int)fields.size(), in.data(), fields.data(),
                                        numTimeSteps, deltaTime, sums.data()),
          "fdb_upwind_advect_host_stream");
    return sums;
  }

  void setArith(int arith, int temporalDepth = 0) {
    check(fdb_upwind_set_arith(h_, arith, temporalDepth), "fdb_upwind_set_arith");
  }

  // FDB_COEFF_CXX or FDB_COEFF_PRODUCT (fdb_upwind_set_coeff_form).
  void setCoeffForm(int form) {
    check(fdb_upwind_set_coeff_form(h_, form), "fdb_upwind_set_coeff_form");
  }

  fdb_upwind* handle() { return h_; }
  size_t size() const { return ntot_; }

 private:
  void create() {
    if (v_.size() < NDIMS || lengths_.size() < NDIMS || numCells_.size() < NDIMS)
      throw std::invalid_argument("Upwind: need NDIMS velocity, lengths and numCells entries");
    std::vector<uint64_t> n(numCells_.begin(), numCells_.begin() + NDIMS);
    check(fdb_upwind_create((int)NDIMS, v_.data(), lengths_.data(), n.data(), &h_),
          "fdb_upwind_create");
    ntot_ = 1;
    for (size_t j = 0; j < NDIMS; ++j) {
      deltas_.push_back(lengths_[j] / numCells_[j]);
      ntot_ *= numCells_[j];
    }
  }

  void axis(std::fstream& file, const char* label, int k) const {
    file << "\n" << label << " ";
    if (k < 0) {
      file << "1 double\n0.0\n";
      return;
    }
    file << numCells_[k] + 1 << " double\n";
    for (size_t i = 0; i < numCells_[k] + 1; ++i) file << ' ' << 0.0 + deltas_[k] * i;
  }

  fdb_upwind* h_ = nullptr;
  std::vector<double> v_, lengths_, deltas_;
  std::vector<size_t> numCells_;
  size_t ntot_ = 0;
};

}  // namespace fdb

#ifndef FDB_NO_GLOBAL_UPWIND
// Drop-in: code written against the reference's global Upwind<NDIMS>.
using fdb::Upwind;
#endif

#endif  // FIDIBENCH_GB_UPWIND_H
