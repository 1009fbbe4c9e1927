# Builds oracle/_ref/libref_tetmesh.so from the reference's own sources where they lie
# (its TetMesh and TriMesh readers and neighbour builders: src/core/cuda/tetmesh.cu,
# src/core/aggmis/cuda/TriMesh_io.cu and TriMesh_connectivity.cu, host code compiled by
# nvcc as the reference's .cu files are) plus the C shim in oracle/ref_shim/.  The rest of
# the reference (assembly, AMG, solver) needs CUSP and cannot be built here.
# Usage: make -f oracle/ref.mk REF=<reference checkout>
REF ?= /root/reference
NVCC ?= nvcc
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref

all: $(OUT)/libref_tetmesh.so

REFSRC := $(REF)/src/core/cuda/tetmesh.cu $(REF)/src/core/aggmis/cuda/TriMesh_io.cu \
          $(REF)/src/core/aggmis/cuda/TriMesh_connectivity.cu
INC := -I $(REF)/src/core/include -I $(REF)/src/core/aggmis/include
FLAGS := -std=c++14 -O2 -Xcompiler -fPIC -w

$(OUT)/libref_tetmesh.so: $(REFSRC) $(HERE)ref_shim/tetmesh_shim.cpp
	mkdir -p $(OUT)
	$(NVCC) $(FLAGS) $(INC) -c $(REF)/src/core/cuda/tetmesh.cu -o $(OUT)/tetmesh.o
	$(NVCC) $(FLAGS) $(INC) -c $(REF)/src/core/aggmis/cuda/TriMesh_io.cu -o $(OUT)/TriMesh_io.o
	$(NVCC) $(FLAGS) $(INC) -c $(REF)/src/core/aggmis/cuda/TriMesh_connectivity.cu -o $(OUT)/TriMesh_connectivity.o
	$(NVCC) $(FLAGS) $(INC) -x cu -c $(HERE)ref_shim/tetmesh_shim.cpp -o $(OUT)/tetmesh_shim.o
	$(NVCC) -shared -o $@ $(OUT)/tetmesh.o $(OUT)/TriMesh_io.o $(OUT)/TriMesh_connectivity.o $(OUT)/tetmesh_shim.o

clean:
	rm -rf $(OUT)

.PHONY: all clean
