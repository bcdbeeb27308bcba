// Shadow of the reference's core/ConfigVariables.hpp, placed ahead of the
// reference's core/ directory on the include path when oracle/Makefile builds
// oracle/_ref/libsphref.so.  It keeps the reference's macro names but turns the
// physics constants into run-time variables owned by ref_harness.cpp, so one
// build of the reference's classes serves every smoothing length and constant
// set used by the golden fixtures.  FP64 build (DOUBLE_PRECISION=ON).
#pragma once

using Real = double;

extern double sphref_H;
extern double sphref_GAS_CONSTANT;
extern double sphref_RHO_0;
extern double sphref_MU;

#define H sphref_H
#define D 2
#define TOL 1.0e-12
#define GAS_CONSTANT sphref_GAS_CONSTANT
#define RHO_0 sphref_RHO_0
#define MU sphref_MU
#define DT 0.01

#define CONFIG_DIR "./"
