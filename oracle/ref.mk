# Builds the reference Blend2D library (portable "fixed" pipeline, no JIT) straight from its
# sources with g++, plus the scene replay harness `ref_replay.cpp` linked against it.
#
# This is test infrastructure only: the outputs land in oracle/_ref/ (git-ignored) and are used
# to generate and check golden vectors. Nothing in the product links against them.
#
#   make -f oracle/ref.mk REF=/root/reference VARIANT=default -j8
#
# VARIANT selects which gradient-LUT builder the reference picks at run time
# (blend2d/pixelops/funcs.cpp:22-34). The library is always built in the default x86-64
# configuration (-DBL_BUILD_OPT_AVX512, which cascades to AVX2/SSE*); only the selector
# translation unit pixelops/funcs.cpp may be compiled with a reduced BL_BUILD_OPT_* set:
#   default - the stock x86-64 no-JIT build. Without asmjit the runtime never detects CPU
#             features (blend2d/core/runtime.cpp:127-180), so the SSE2 builder is selected;
#   scalar  - funcs.cpp sees no BL_BUILD_OPT_* (the portable interpolate_prgb32, which is what
#             a no-JIT build on a non-x86 host selects).
# b2d_reflut calls all three builders (scalar, SSE2, AVX2) directly for LUT known answers.
# Compiler flags follow CMakeLists.txt:645-680 (GNU branch) and the per-file ISA flags at
# CMakeLists.txt:725-734. x86-64 hosts only.

REF      ?= /root/reference
VARIANT  ?= default
HERE     := $(dir $(lastword $(MAKEFILE_LIST)))
OUT      := $(HERE)_ref
OBJ      := $(OUT)/obj_$(VARIANT)
CXX      ?= g++

OPT_DEFS := -DBL_BUILD_OPT_AVX512
ifeq ($(VARIANT),default)
  FUNCS_DEFS := -DBL_BUILD_OPT_AVX512
else ifeq ($(VARIANT),scalar)
  FUNCS_DEFS :=
else
  $(error unknown VARIANT $(VARIANT))
endif

CXXFLAGS := -std=c++17 -O2 -fPIC -fno-math-errno -fno-threadsafe-statics -fno-exceptions -fno-rtti \
            -fmerge-all-constants -fno-semantic-interposition -fno-trapping-math -fno-finite-math-only \
            -ftree-vectorize -fvisibility=hidden -DBL_STATIC -DBL_BUILD_NO_JIT -I$(REF) -w

SRCS := $(shell cd $(REF) && find blend2d -name '*.cpp' ! -name '*_test.cpp' ! -path '*/jit/*' | sort)
OBJS := $(patsubst %.cpp,$(OBJ)/%.o,$(SRCS))

# Per-file ISA flags (CMakeLists.txt:725-734); files for ISAs the variant does not enable still
# compile (their bodies are guarded by BL_TARGET_OPT_* checks) and register nothing.
isa_flags = $(strip \
  $(if $(filter %_sse3.cpp,$1),-msse3) \
  $(if $(filter %_ssse3.cpp,$1),-mssse3) \
  $(if $(filter %_sse4_1.cpp,$1),-msse4.1) \
  $(if $(filter %_sse4_2.cpp,$1),-mpopcnt -mpclmul -msse4.2) \
  $(if $(filter %_avx.cpp,$1),-mpopcnt -mpclmul -mavx) \
  $(if $(filter %_avx2.cpp,$1),-mpopcnt -mpclmul -mbmi -mbmi2 -mavx2 -DBL_TARGET_OPT_POPCNT -DBL_TARGET_OPT_BMI2) \
  $(if $(filter %_avx512.cpp,$1),-mpopcnt -mpclmul -mbmi -mbmi2 -mavx512f -mavx512bw -mavx512dq -mavx512cd -mavx512vl -DBL_TARGET_OPT_POPCNT -DBL_TARGET_OPT_BMI2))

LIB    := $(OUT)/libblend2d_$(VARIANT).a
REPLAY := $(OUT)/b2d_replay_$(VARIANT)

REFLUT := $(OUT)/b2d_reflut
REFRAS := $(OUT)/b2d_refras

all: $(REPLAY) $(if $(filter default,$(VARIANT)),$(REFLUT) $(REFRAS))

$(OBJ)/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(if $(filter %pixelops/funcs.cpp,$<),$(FUNCS_DEFS),$(OPT_DEFS)) $(call isa_flags,$<) -c $< -o $@

$(LIB): $(OBJS)
	rm -f $@
	ar rcs $@ $(OBJS)

$(REPLAY): $(HERE)ref_replay.cpp $(HERE)../include/blgpu_stream.h $(LIB)
	$(CXX) -std=c++17 -O2 -DBL_STATIC -I$(REF) -I$(HERE)../include $(HERE)ref_replay.cpp $(LIB) -lpthread -lrt -o $@

$(REFLUT): $(HERE)ref_lut.cpp $(LIB)
	$(CXX) -std=c++17 -O2 -DBL_STATIC -I$(REF) $(HERE)ref_lut.cpp $(LIB) -lpthread -lrt -o $@

$(REFRAS): $(HERE)ref_raster.cpp $(LIB)
	$(CXX) -std=c++17 -O2 -DBL_STATIC -DBL_BUILD_NO_JIT -I$(REF) $(HERE)ref_raster.cpp $(LIB) -lpthread -lrt -o $@

.PHONY: all
