# Builds oracle/_ref/libref_tetmesh.so from the reference's own sources where they lie
# (its TetMesh reader and neighbour builder, src/core/cuda/tetmesh.cu, host code compiled
# by nvcc as the reference's .cu files are) plus the C shim in oracle/ref_shim/.  The rest
# of the reference (assembly, AMG, solver) needs CUSP and cannot be built here.
# Usage: make -f oracle/ref.mk REF=<reference checkout>
REF ?= /root/reference
NVCC ?= nvcc
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref

all: $(OUT)/libref_tetmesh.so

$(OUT)/libref_tetmesh.so: $(REF)/src/core/cuda/tetmesh.cu $(HERE)ref_shim/tetmesh_shim.cpp
	mkdir -p $(OUT)
	$(NVCC) -std=c++14 -O2 -Xcompiler -fPIC -I $(REF)/src/core/include -c $(REF)/src/core/cuda/tetmesh.cu -o $(OUT)/tetmesh.o -w
	$(NVCC) -std=c++14 -O2 -Xcompiler -fPIC -I $(REF)/src/core/include -x cu -c $(HERE)ref_shim/tetmesh_shim.cpp -o $(OUT)/tetmesh_shim.o -w
	$(NVCC) -shared -o $@ $(OUT)/tetmesh.o $(OUT)/tetmesh_shim.o

clean:
	rm -rf $(OUT)

.PHONY: all clean
