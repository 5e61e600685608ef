// upwindAcc2Cxx -- the reference's upwindAcc2 driver (upwind/cxx/upwindAcc2.cxx,
// one advect(numSteps, dt) call, -std) on the GB300 library (acc_driver.h).
#include "acc_driver.h"

int main(int argc, char** argv) { return fdb_drivers::run_acc_driver(argc, argv, false); }
