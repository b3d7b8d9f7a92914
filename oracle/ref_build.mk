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
#   make -f oracle/ref_build.mk REF=<IMSRG++ checkout> -j8
#   make -f oracle/ref_build.mk REF=<checkout> SCIPY_OPENBLAS=<libscipy_openblas .so> blas -j8
#
# REF defaults to the environment variable IMSRG_REFERENCE.

REF ?= $(IMSRG_REFERENCE)
ifeq ($(strip $(REF)),)
$(error set REF (or IMSRG_REFERENCE) to the IMSRG++ checkout)
endif
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

# The same closure with Armadillo's BLAS path on (LAPACK stays off: the path
# calls none), BLAS from SciPy's OpenBLAS through ref_stubs/blas_forward.c:
# the reference as its own build runs it, for timing against the C oracle.
# Built only on request (target blas).
SCIPY_OPENBLAS ?=
OBJB := $(OUT)/obj_blas
DEFS_BLAS := -DARMA_DONT_USE_WRAPPER -DARMA_DONT_USE_LAPACK -DARMA_NO_DEBUG -DNO_ODE
CXXFLAGS_BLAS := -std=c++17 -O2 -fopenmp -w $(DEFS_BLAS) $(INCS)
REF_OBJS_BLAS := $(addprefix $(OBJB)/,$(addsuffix .o,$(REF_UNITS)))

blas: $(OUT)/ref_harness_blas

$(OBJB):
	mkdir -p $(OBJB)

$(OBJB)/%.o: $(SRC)/%.cc | $(OBJB)
	$(CXX) $(CXXFLAGS_BLAS) -c $< -o $@

$(OBJB)/ode_stub.o: $(ORACLE)ref_stubs/ode_stub.cc | $(OBJB)
	$(CXX) $(CXXFLAGS_BLAS) -c $< -o $@

$(OBJB)/ref_harness.o: $(ORACLE)ref_harness.cc | $(OBJB)
	$(CXX) $(CXXFLAGS_BLAS) -c $< -o $@

$(OBJB)/blas_forward.o: $(ORACLE)ref_stubs/blas_forward.c | $(OBJB)
	$(CC) -O2 -fPIC -c $< -o $@

$(OUT)/ref_harness_blas: $(REF_OBJS_BLAS) $(OBJ)/coupling_stub.o $(OBJB)/ode_stub.o $(OBJB)/ref_harness.o \
		$(OBJB)/blas_forward.o
	@test -n "$(SCIPY_OPENBLAS)" || (echo "set SCIPY_OPENBLAS to SciPy's libscipy_openblas .so" && false)
	$(CXX) -fopenmp -o $@ $^ $(SCIPY_OPENBLAS) -Wl,-rpath,$(dir $(SCIPY_OPENBLAS)) -lm

# The drop-in link: imsrg_gb300/shim/imsrg_gpu_shim.cc in place of the
# reference's IMSRG(2) terms, CommutatorScalarScalar and
# Standard_BCH_Transform.  Copies of Commutator.o and BCH.o get those symbols
# made weak (objcopy), so the shim's definitions are the ones linked; every
# other object is the reference's own.  Needs the built library (LIB).
# Built only on request (target shim); oracle/shim_harness.cc is the driver.
REPO := $(abspath $(ORACLE)..)
LIB ?= $(REPO)/imsrg_gb300/_build/libimsrg_gb300.so
SHIM_COMM_SYMS := _ZN10Commutator9comm110ssERK8OperatorS2_RS0_ _ZN10Commutator9comm220ssERK8OperatorS2_RS0_ \
  _ZN10Commutator9comm111ssERK8OperatorS2_RS0_ _ZN10Commutator9comm121ssERK8OperatorS2_RS0_ \
  _ZN10Commutator9comm122ssERK8OperatorS2_RS0_ _ZN10Commutator9comm221ssERK8OperatorS2_RS0_ \
  _ZN10Commutator15comm222_pp_hhssERK8OperatorS2_RS0_ _ZN10Commutator19comm222_pp_hh_221ssERK8OperatorS2_RS0_ \
  _ZN10Commutator12comm222_phssERK8OperatorS2_RS0_ _ZN10Commutator22CommutatorScalarScalarERK8OperatorS2_
SHIM_BCH_SYMS := _ZN3BCH22Standard_BCH_TransformERK8OperatorS2_
SHIM_BASE_OBJS := $(filter-out $(OBJ)/Commutator.o $(OBJ)/BCH.o,$(REF_OBJS))

shim: $(OUT)/shim_harness

$(OBJ)/Commutator_weak.o: $(OBJ)/Commutator.o
	objcopy $(addprefix --weaken-symbol=,$(SHIM_COMM_SYMS)) $< $@

$(OBJ)/BCH_weak.o: $(OBJ)/BCH.o
	objcopy $(addprefix --weaken-symbol=,$(SHIM_BCH_SYMS)) $< $@

$(OBJ)/imsrg_gpu_shim.o: $(REPO)/imsrg_gb300/shim/imsrg_gpu_shim.cc $(REPO)/include/imsrg_gb300.h | $(OBJ)
	$(CXX) $(CXXFLAGS) -I$(REPO)/include -c $< -o $@

$(OBJ)/shim_harness.o: $(ORACLE)shim_harness.cc | $(OBJ)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/shim_harness: $(SHIM_BASE_OBJS) $(OBJ)/Commutator_weak.o $(OBJ)/BCH_weak.o $(OBJ)/imsrg_gpu_shim.o \
		$(OBJ)/coupling_stub.o $(OBJ)/ode_stub.o $(OBJ)/shim_harness.o $(LIB)
	$(CXX) -fopenmp -o $@ $^ -Wl,-rpath,$(dir $(LIB)) -lm

clean:
	rm -rf $(OUT)/obj $(OUT)/obj_blas $(OUT)/ref_harness $(OUT)/ref_harness_blas $(OUT)/shim_harness

.PHONY: all blas shim clean
