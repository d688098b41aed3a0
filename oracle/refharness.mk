# Build of the reference's own CUDA path under a non-MATLAB harness
# (refharness.cu) against the headers staged by stage_reference.sh into
# _ref/src.  Outputs go to _ref/ only.  One binary per DIMS.
NVCC ?= /usr/local/cuda/bin/nvcc
REF  := _ref/src
OUT  := _ref
FLAGS := -std=c++17 -O2 -gencode arch=compute_103a,code=sm_103a -I $(REF)

all: $(OUT)/refharness2d $(OUT)/refharness3d

$(OUT)/refharness2d: refharness.cu $(REF)/Simulation.cuh
	$(NVCC) $(FLAGS) -DDIMS=2 refharness.cu -lcublas -o $@

$(OUT)/refharness3d: refharness.cu $(REF)/Simulation.cuh
	$(NVCC) $(FLAGS) -DDIMS=3 refharness.cu -lcublas -o $@

.PHONY: all
