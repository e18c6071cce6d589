# The reference's own CUDA path (microLC simulating_lcurves: gpu_functions.cu with its cuFFT
# expanding_source, thrust z-sort and pair kernels; data_structs.cu; the CPU files they call)
# built unchanged for sm_103a with a small C entry layer (oracle/ref_cuda_harness.cu), as a
# parity pin and a timed baseline on the GPU.  Test infrastructure only.
#
#   make -f oracle/refcuda.mk stage REF=<reference checkout>/simulating_lcurves
#       copies the sources it needs into baseline/_ref/microlc (git-ignored: the reference
#       installed beside the repository, which travels with it to a GPU machine where the
#       reference checkout does not exist);
#   make -f oracle/refcuda.mk
#       compiles that copy into baseline/_ref/libmlcref_cuda.so.
#
# The reference's headers include <png.h> and <CCfits/CCfits> for image writers that are
# not on this path: empty stand-ins are generated.  Its configure script passes no
# -arch/-gencode; here the one GPU target is sm_103a.  No source file is changed.

ROOT     := $(abspath $(dir $(lastword $(MAKEFILE_LIST)))/..)
OUT      := $(ROOT)/baseline/_ref
SRC      := $(OUT)/microlc
CUDA     ?= /usr/local/cuda
NVCC     ?= $(CUDA)/bin/nvcc
FILES    := src/gpu_functions.cu src/data_structs.cu src/util.cu src/profile.cpp src/magnification_map.cpp \
            src/cpu_functions.cpp src/mpd.cpp src/integration.cpp src/locations.cpp
FLAGS    := -std=c++17 -O2 -gencode arch=compute_103a,code=sm_103a -Xcompiler -fPIC -w \
            -I$(OUT)/stubs -I$(SRC)/include -DMAP_PATH='""'
OBJS     := $(addprefix $(OUT)/obj/,$(notdir $(addsuffix .o,$(FILES)))) $(OUT)/obj/ref_cuda_harness.cu.o

all: $(OUT)/libmlcref_cuda.so

stage:
	@test -n "$(REF)" || (echo "set REF=<reference checkout>/simulating_lcurves" && exit 2)
	mkdir -p $(SRC)/src $(SRC)/include
	cp $(addprefix $(REF)/,$(FILES)) $(SRC)/src/
	cp $(REF)/include/*.hpp $(SRC)/include/

$(OUT)/stubs/png.h:
	mkdir -p $(OUT)/stubs/CCfits
	printf '/* empty stand-in: image writers are not built */\n' > $(OUT)/stubs/png.h
	printf '#include <vector>\n#include <valarray>\n#include <memory>\n' > $(OUT)/stubs/CCfits/CCfits

$(OUT)/obj/%.cu.o: $(SRC)/src/%.cu $(OUT)/stubs/png.h
	mkdir -p $(OUT)/obj
	$(NVCC) $(FLAGS) -c $< -o $@

$(OUT)/obj/%.cpp.o: $(SRC)/src/%.cpp $(OUT)/stubs/png.h
	mkdir -p $(OUT)/obj
	$(NVCC) $(FLAGS) -x cu -c $< -o $@

$(OUT)/obj/ref_cuda_harness.cu.o: $(ROOT)/oracle/ref_cuda_harness.cu $(OUT)/stubs/png.h
	mkdir -p $(OUT)/obj
	$(NVCC) $(FLAGS) -c $< -o $@

$(OUT)/libmlcref_cuda.so: $(OBJS)
	$(NVCC) -shared -gencode arch=compute_103a,code=sm_103a -o $@ $^ -lcufft

.PHONY: all stage
