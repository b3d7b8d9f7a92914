# Test infrastructure: NOT part of the product.
#
# Compiles the reference implementation (IMSRG++) from its own, unmodified
# sources where they lie, plus the stand-ins in oracle/ref_stubs/ for the
# libraries this image lacks (GSL coupling coefficients, Boost iostreams, the
# Boost odeint solvers of IMSRGSolver), and
# links oracle/ref_harness.cc against them.  Armadillo is the copy vendored in
# the reference (extern/armadillo); BLAS/LAPACK are not installed, so Armadillo
# runs on its built-in matrix product (ARMA_DONT_USE_BLAS / _LAPACK / _WRAPPER).
# Every output goes to oracle/_ref/.  Used only in the build container (the
# reference sources do not exist elsewhere).
#
#   make -f oracle/ref_build.mk [REF=/root/reference] -j8

REF ?= /root/reference
SRC := $(REF)/src
ORACLE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(ORACLE)_ref
OBJ := $(OUT)/obj

CXX ?= g++
CC ?= gcc
DEFS := -DARMA_DONT_USE_WRAPPER -DARMA_DONT_USE_BLAS -DARMA_DONT_USE_LAPACK -DARMA_NO_DEBUG -DNO_ODE
INCS := -I$(ORACLE)ref_stubs -I$(SRC) -I$(REF)/extern/armadillo -I$(REF)/extern/half/include
CXXFLAGS := -std=c++17 -O2 -fopenmp -w $(DEFS) $(INCS)

# the closure of the IMSRG(2) commutator + BCH path and the Magnus solver (the three-body, tensor and
# dagger objects only satisfy references from Commutator.cc / Operator.cc)
REF_UNITS := AngMom AngMomCache ModelSpace TwoBodyChannel TwoBodyME Operator \
  Commutator BCH IMSRGProfiler ThreeBodyME ThreeBodyChannel ThreeBodyStorage \
  ThreeBodyStorage_pn ThreeBodyStorage_iso ThreeBodyStorage_no2b ThreeBodyStorage_mono \
  ThreeLegME IMSRG3Commutators Commutator232 TensorCommutators DaggerCommutators \
  FactorizedDoubleCommutator ReferenceImplementations Generator IMSRGSolver version

REF_OBJS := $(addprefix $(OBJ)/,$(addsuffix .o,$(REF_UNITS)))

all: $(OUT)/ref_harness

$(OBJ):
	mkdir -p $(OBJ)

$(OBJ)/%.o: $(SRC)/%.cc | $(OBJ)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/coupling_stub.o: $(ORACLE)ref_stubs/coupling_stub.c | $(OBJ)
	$(CC) -O2 -fPIC -c $< -o $@

$(OBJ)/ode_stub.o: $(ORACLE)ref_stubs/ode_stub.cc | $(OBJ)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/ref_harness.o: $(ORACLE)ref_harness.cc | $(OBJ)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/ref_harness: $(REF_OBJS) $(OBJ)/coupling_stub.o $(OBJ)/ode_stub.o $(OBJ)/ref_harness.o
	$(CXX) -fopenmp -o $@ $^ -lm

clean:
	rm -rf $(OUT)/obj $(OUT)/ref_harness

.PHONY: all clean
