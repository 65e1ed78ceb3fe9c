# Compiles the reference AMDAT program from its own sources, where they lie,
# into OUT (object files, a generated version header, an FFTW stub header, the
# extracted q-vector tables and the AMDAT binary).  Nothing is written into the
# reference tree.  Usage (from the repository root):
#   make -f oracle/ref.mk REF=/path/to/AMDAT OUT=oracle/_ref/<machine> -j8
# (oracle/build_oracle.py runs it).  The reference is used only as the parity
# checker and the benchmark's CPU reference.
ifndef REF
$(error REF must name the AMDAT source tree)
endif
OUT     ?= oracle/_ref/$(shell uname -m)
CXX     ?= g++
CC      ?= gcc
SEMVER  := $(strip $(shell cat $(REF)/VERSION 2>/dev/null || echo 0.0.0))
QV      := $(abspath $(OUT))/qvectors
# The reference's Makefile also excludes these three translation units.
EXCLUDE := time_correlation_function.cpp spherical_wave_vectors.cpp spacial_decomposition.cpp
SRCS    := $(filter-out $(addprefix $(REF)/src/,$(EXCLUDE)),$(wildcard $(REF)/src/*.cpp))
OBJS    := $(patsubst $(REF)/src/%.cpp,$(OUT)/obj/%.o,$(SRCS))
XDR     := xdrfile xdrfile_xtc xdrfile_trr
XOBJS   := $(addprefix $(OUT)/obj/xdr_,$(addsuffix .o,$(XDR)))
# -D_FORTIFY_SOURCE=0: Wave_Vectors::read_vectors writes 5 bytes into char[4]
# (wave_vectors.cpp:431/443), which glibc's fortified sprintf aborts on.
CXXFLAGS := -std=c++17 -O3 -DNDEBUG -fopenmp -w -U_FORTIFY_SOURCE -D_FORTIFY_SOURCE=0 \
  -I$(REF)/src -I$(OUT)/gen -I$(OUT)/gen/generated \
  -I$(REF)/third_party/voro++-0.4.6/src -I$(REF)/third_party/xdrfile-1.1b/include \
  -I$(REF)/third_party/xdrfile-1.1b \
  -DWV3D='"$(QV)/qvectors3d/qvector"' -DWV2D='"$(QV)/qvectors2d/qvector"' \
  -DWV1D='"$(QV)/qvectors1d/qvector"'
CFLAGS  := -O3 -w -I$(REF)/third_party/xdrfile-1.1b/include

all: $(OUT)/AMDAT

$(OUT)/gen/generated/version.h:
	@mkdir -p $(dir $@)
	@printf '#pragma once\nnamespace amdat::build {\ninline constexpr const char* NAME="AMDAT";\ninline constexpr const char* SEMVER="%s";\ninline constexpr const char* GIT_DESCRIBE="";\ninline constexpr const char* GIT_COMMIT="";\ninline constexpr const char* GIT_BRANCH="";\ninline constexpr const char* BUILD_DATE="";\ninline constexpr const char* COMPILER="gcc";\ninline constexpr bool OPENMP=true;\n}\n' '$(SEMVER)' > $@

# FFTW is not installed; only the vac_fourier command uses it.  This stub
# declares the four calls so the unit compiles; calling them aborts.
$(OUT)/gen/fftw3.h:
	@mkdir -p $(dir $@)
	@printf '#pragma once\n#include <stdlib.h>\ntypedef double fftw_complex[2];\ntypedef void* fftw_plan;\n#define FFTW_ESTIMATE 0\nstatic inline void* fftw_malloc(size_t n){(void)n; abort();}\nstatic inline fftw_plan fftw_plan_dft_r2c_1d(int n,double*i,fftw_complex*o,unsigned f){(void)n;(void)i;(void)o;(void)f; abort();}\nstatic inline void fftw_execute(fftw_plan p){(void)p; abort();}\nstatic inline void fftw_destroy_plan(fftw_plan p){(void)p;}\nstatic inline void fftw_free(void*p){(void)p;}\n' > $@

$(OUT)/qvectors/.ready:
	@mkdir -p $(OUT)/qvectors
	python3 -c "import zipfile,sys; zipfile.ZipFile(sys.argv[1]).extractall(sys.argv[2])" $(REF)/src/qvectors/qvectors.zip $(OUT)/qvectors
	@touch $@

$(OUT)/obj/%.o: $(REF)/src/%.cpp $(OUT)/gen/generated/version.h $(OUT)/gen/fftw3.h
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/obj/xdr_%.o: $(REF)/third_party/xdrfile-1.1b/src/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) -c $< -o $@

$(OUT)/obj/voro.o: $(REF)/third_party/voro++-0.4.6/src/voro++.cc
	@mkdir -p $(dir $@)
	$(CXX) -O3 -w -c $< -o $@

$(OUT)/AMDAT: $(OBJS) $(XOBJS) $(OUT)/obj/voro.o $(OUT)/qvectors/.ready
	$(CXX) -fopenmp -o $@ $(OBJS) $(XOBJS) $(OUT)/obj/voro.o -lm

.PHONY: all
