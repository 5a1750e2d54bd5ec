# Builds the reference Blend2D library (portable "fixed" pipeline, no JIT) straight from its
# sources with g++, plus the scene replay harness `ref_replay.cpp` linked against it.
#
# This is test infrastructure only: the outputs land in oracle/_ref/ (git-ignored) and are used
# to generate and check golden vectors and, in bench.py's reference arm, as the CPU baseline.
# Nothing in the product links against them.
#
#   make -f oracle/ref.mk REF=<reference checkout> VARIANT=default -j8
#
# REF defaults to the copy of the reference's library sources that oracle/stage_ref.sh places in
# baseline/_ref/blend2d-src (git-ignored; it travels with the repository to hosts that have no
# reference checkout).
#
# VARIANT selects the host and which gradient-LUT builder the reference picks at run time
# (blend2d/pixelops/funcs.cpp:22-34):
#   default - x86-64: the stock no-JIT build (-DBL_BUILD_OPT_AVX512, which cascades to
#             AVX2/SSE*). Without asmjit the runtime never detects CPU features
#             (blend2d/core/runtime.cpp:127-180), so the SSE2 builder is selected;
#   scalar  - x86-64, but pixelops/funcs.cpp sees no BL_BUILD_OPT_* (the portable
#             interpolate_prgb32, which is what a no-JIT build on a non-x86 host selects);
#   native  - any other host (the aarch64 GPU hosts): no ISA flags at all, the portable LUT
#             builder, and -ffp-contract=off so that GCC does not fuse a*b+c into FMAs on a
#             target where it otherwise would (the reference's arithmetic, as its x86-64 baseline
#             build evaluates it).
# b2d_reflut calls all three builders (scalar, SSE2, AVX2) directly for LUT known answers.
# Compiler flags follow CMakeLists.txt:645-680 (GNU branch) and the per-file ISA flags at
# CMakeLists.txt:725-734.

HERE     := $(dir $(lastword $(MAKEFILE_LIST)))
REF      ?= $(HERE)../baseline/_ref/blend2d-src
VARIANT  ?= default
OUT      := $(HERE)_ref
OBJ      := $(OUT)/obj_$(VARIANT)
CXX      ?= g++

ifeq ($(VARIANT),default)
  OPT_DEFS   := -DBL_BUILD_OPT_AVX512
  FUNCS_DEFS := -DBL_BUILD_OPT_AVX512
  X86        := 1
else ifeq ($(VARIANT),scalar)
  OPT_DEFS   := -DBL_BUILD_OPT_AVX512
  FUNCS_DEFS :=
  X86        := 1
else ifeq ($(VARIANT),native)
  OPT_DEFS   := -ffp-contract=off
  FUNCS_DEFS := -ffp-contract=off
  X86        :=
else
  $(error unknown VARIANT $(VARIANT))
endif

CXXFLAGS := -std=c++17 -O2 -fPIC -fno-math-errno -fno-threadsafe-statics -fno-exceptions -fno-rtti \
            -fmerge-all-constants -fno-semantic-interposition -fno-trapping-math -fno-finite-math-only \
            -ftree-vectorize -fvisibility=hidden -DBL_STATIC -DBL_BUILD_NO_JIT -I$(REF) -w

SRCS := $(shell cd $(REF) && find blend2d -name '*.cpp' ! -name '*_test.cpp' ! -path '*/jit/*' | sort)
OBJS := $(patsubst %.cpp,$(OBJ)/%.o,$(SRCS))

# Per-file ISA flags (CMakeLists.txt:725-734); files for ISAs the variant does not enable still
# compile (their bodies are guarded by BL_TARGET_OPT_* checks) and register nothing. The native
# variant passes none.
isa_flags = $(if $(X86),$(isa_flags_x86))
isa_flags_x86 = $(strip \
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

# The replay harness alone (what bench.py's reference arm and the GPU host's tests need).
replay: $(REPLAY)

# The BLContext binding (blend2d_gb300/blcontext) linked with this reference library and
# libblgpu.so (built first by blend2d_gb300/build.py), with its check harness.
BLGPU_LIB := $(HERE)../blend2d_gb300/_build
BLCONTEXT := $(OUT)/b2d_blcontext_$(VARIANT)
blcontext: $(BLCONTEXT)

$(BLCONTEXT): $(HERE)../tests/native/blcontext_check.cpp $(HERE)../blend2d_gb300/blcontext/blgpu_blcontext.cpp \
              $(HERE)../include/blgpu_blcontext.h $(HERE)../include/blgpu.h $(HERE)ref_stream.h $(LIB) $(BLGPU_LIB)/libblgpu.so
	$(CXX) -std=c++17 -O2 -ffp-contract=off -DBL_STATIC -I$(REF) -I$(HERE)../include \
	  $(HERE)../tests/native/blcontext_check.cpp $(HERE)../blend2d_gb300/blcontext/blgpu_blcontext.cpp $(LIB) \
	  -L$(BLGPU_LIB) -lblgpu -Wl,-rpath,'$$ORIGIN/../../blend2d_gb300/_build' -lpthread -lrt -o $@

$(OBJ)/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(if $(filter %pixelops/funcs.cpp,$<),$(FUNCS_DEFS),$(OPT_DEFS)) $(call isa_flags,$<) -c $< -o $@

$(LIB): $(OBJS)
	rm -f $@
	ar rcs $@ $(OBJS)

$(REPLAY): $(HERE)ref_replay.cpp $(HERE)ref_stream.h $(HERE)../include/blgpu_stream.h $(LIB)
	$(CXX) -std=c++17 -O2 -ffp-contract=off -DBL_STATIC -I$(REF) -I$(HERE)../include $(HERE)ref_replay.cpp $(LIB) -lpthread -lrt -o $@

$(REFLUT): $(HERE)ref_lut.cpp $(LIB)
	$(CXX) -std=c++17 -O2 -DBL_STATIC -I$(REF) $(HERE)ref_lut.cpp $(LIB) -lpthread -lrt -o $@

$(REFRAS): $(HERE)ref_raster.cpp $(LIB)
	$(CXX) -std=c++17 -O2 -DBL_STATIC -DBL_BUILD_NO_JIT -I$(REF) $(HERE)ref_raster.cpp $(LIB) -lpthread -lrt -o $@

.PHONY: all replay blcontext
