# Test infrastructure only.  Compiles the reference's CARE correction sources
# where they lie (never copied into this repository) plus this directory's
# drivers, writing every output under oracle/_ref/.  Usage:
#     make -f oracle/ref.mk REF=/path/to/RabbitQCPlus -j8
# (REF has no default: oracle.build_reference passes it.)
# The reference's own Makefile is not used: these are the few translation
# units that care::performCorrection needs, built with the reference's own
# language/optimisation flags (ISO C++17, so floating-point contraction is off,
# -O3, OpenMP, thrust on its OpenMP backend).  No -march=native: the SIMD block
# guarded by Vec512 in src/cpu_alignment.cpp is unused by the selected path.

ifndef REF
$(error REF (the reference source tree) is not set)
endif
OUT := oracle/_ref
OBJ := $(OUT)/obj
CXX ?= g++

REF_SRCS := dispatch_care_correct_cpu correct_cpu msa cpu_alignment \
            cpuminhasherconstruction options readlibraryio \
            correctionresultoutput threadpool

CXXFLAGS := -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP \
            -fconstexpr-ops-limit=99000100 -DNDUBUG -std=c++17 \
            -I$(REF) -I$(REF)/common -I$(REF)/include -I$(REF)/include/huffman \
            -I$(REF)/include/chunkdecoding -I$(REF)/include/gzip \
            -I$(REF)/src/include -I$(REF)/dependencies/thrust-1.17.0 \
            -O3 -w -fopenmp -ffp-contract=off
LIBS := -lpthread -fopenmp -lrt -lgomp -lstdc++fs -lz -ldl

REF_OBJS := $(patsubst %,$(OBJ)/%.o,$(REF_SRCS))

all: $(OUT)/ref_care $(OUT)/ref_stages

$(OBJ)/%.o: $(REF)/src/%.cpp
	@mkdir -p $(OBJ)
	$(CXX) -c $< -o $@ $(CXXFLAGS)

$(OBJ)/ref_driver.o: oracle/ref_driver.cpp
	@mkdir -p $(OBJ)
	$(CXX) -c $< -o $@ $(CXXFLAGS)

$(OBJ)/ref_stages.o: oracle/ref_stages.cpp
	@mkdir -p $(OBJ)
	$(CXX) -c $< -o $@ $(CXXFLAGS)

$(OUT)/ref_care: $(REF_OBJS) $(OBJ)/ref_driver.o
	$(CXX) $^ -o $@ $(LIBS)

# ref_stages builds its own read store/minhasher, so it leaves out the dispatch
# object (whose header-defined constructChunkedReadStorageFromFiles would clash).
$(OUT)/ref_stages: $(filter-out $(OBJ)/dispatch_care_correct_cpu.o,$(REF_OBJS)) $(OBJ)/ref_stages.o
	$(CXX) $^ -o $@ $(LIBS)

.PHONY: all

# The drop-in check: RabbitQCPlus's own caller (main_correction,
# src/main_correct_cpu.cpp) and CARE objects, with dispatch_care_correct_cpu.o
# replaced by the GB300 shim, linked against libcaregpu.so; the driver is
# tests/shim_consumer.cpp.  Needs rabbitqcplus_gb300/lib/libcaregpu.so built.
SHIM := rabbitqcplus_gb300/csrc/host/dispatch_care_correct_gpu.cpp
GPULIB := rabbitqcplus_gb300/lib

$(OBJ)/dispatch_care_correct_gpu.o: $(SHIM) rabbitqcplus_gb300/csrc/host/care_host.h include/care_gpu.h
	@mkdir -p $(OBJ)
	$(CXX) -c $< -o $@ $(CXXFLAGS) -Iinclude -Irabbitqcplus_gb300/csrc/host

$(OBJ)/shim_consumer.o: tests/shim_consumer.cpp rabbitqcplus_gb300/csrc/host/care_host.h
	@mkdir -p $(OBJ)
	$(CXX) -c $< -o $@ $(CXXFLAGS) -I$(REF)/src -Iinclude -Irabbitqcplus_gb300/csrc/host

$(OUT)/care_gpu_dropin: $(filter-out $(OBJ)/dispatch_care_correct_cpu.o,$(REF_OBJS)) $(OBJ)/main_correct_cpu.o \
                        $(OBJ)/dispatch_care_correct_gpu.o $(OBJ)/shim_consumer.o $(GPULIB)/libcaregpu.so
	$(CXX) $(filter %.o,$^) -o $@ $(LIBS) -L$(GPULIB) -lcaregpu -Wl,-rpath,$(abspath $(GPULIB))

.PHONY: dropin
dropin: $(OUT)/care_gpu_dropin
