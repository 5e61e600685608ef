// upwindAccCxx -- the reference's upwindAcc driver (upwind/cxx/upwindAcc.cxx,
// one advect(dt) call per time step) on the GB300 library (acc_driver.h).
#include "acc_driver.h"

int main(int argc, char** argv) { return fdb_drivers::run_acc_driver(argc, argv, true); }
