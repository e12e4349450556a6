# Builds the reference's own CPU implementation of the recovery path (ParPar
# gf16/ + hasher/ cores, non-libuv std::future mode) from a reference source
# tree, plus the shims of this folder.  Test infrastructure only: it pins the
# oracle, generates golden fixtures, is the timed CPU path of the benchmark's
# reference arm, and hosts the PAR2ProcCUDA adapter under the reference's own
# PAR2Proc.  Outputs go to oracle/_ref/ (git-ignored).
#
#   make -f oracle/ref.mk REF=<reference tree> ref        # libparref.so
#   make -f oracle/ref.mk REF=<reference tree> ref_cuda   # libparref_cuda.so (needs libpar2cuda.so)
#
# oracle/refsrc.py stages the tree into oracle/_ref/src and calls this recipe.
ifndef REF
$(error REF=<reference source tree> is required)
endif
OUT := oracle/_ref
OBJ := $(OUT)/obj

ARCH := $(shell uname -m)
# ISA flags per file as binding.gyp sets them (binding.gyp:10-21 target
# defaults, :289-420 hasher targets, :765-871 gf16 ARM targets); the
# reference's CPUID dispatch picks the kernels at run time
ifeq ($(ARCH),x86_64)
ISA := -march=native
ISA_CRC := -march=native
ISA_SVE := -march=native
ISA_SVE2 := -march=native
else
ISA := $(shell $(CC) -march=native -E -x c /dev/null >/dev/null 2>&1 && echo -march=native || echo -march=armv8-a+crc)
ISA_CRC := -march=armv8-a+crc
ISA_SVE := $(shell $(CC) -march=armv8-a+sve -E -x c /dev/null >/dev/null 2>&1 && echo -march=armv8-a+sve || echo $(ISA))
ISA_SVE2 := $(shell $(CC) -march=armv8-a+sve2 -E -x c /dev/null >/dev/null 2>&1 && echo -march=armv8-a+sve2 || echo $(ISA))
endif

CRC_FILES := hasher/hasher_armcrc.cpp hasher/hasher_neoncrc.cpp
SVE_FILES := gf16/gf16_shuffle128_sve.c gf16/gf_add_sve.c gf16/gf16_cksum_sve.c
SVE2_FILES := gf16/gf16_shuffle128_sve2.c gf16/gf16_shuffle2x128_sve2.c gf16/gf16_shuffle512_sve2.c \
              gf16/gf16_clmul_sve2.c gf16/gf_add_sve2.c hasher/hasher_sve2.cpp
isa_of = $(if $(filter $(1),$(CRC_FILES)),$(ISA_CRC),$(if $(filter $(1),$(SVE_FILES)),$(ISA_SVE),$(if $(filter $(1),$(SVE2_FILES)),$(ISA_SVE2),$(ISA))))

COMMON := -O3 -fomit-frame-pointer -DNDEBUG -fno-strict-aliasing -fPIC -I$(REF) -Wno-unused-function -w
CFLAGS := $(COMMON) -std=gnu99
CXXFLAGS := $(COMMON) -std=c++11 -fexceptions

GF_C := $(notdir $(wildcard $(REF)/gf16/*.c))
GF_CXX := gf16mul.cpp controller.cpp controller_cpu.cpp
HS_CXX := $(notdir $(wildcard $(REF)/hasher/*.cpp))
SRCS := $(addprefix gf16/,$(GF_C) $(GF_CXX)) $(addprefix hasher/,$(HS_CXX)) hasher/crc_zeropad.c hasher/md5-final.c
REF_OBJS := $(patsubst %,$(OBJ)/%.o,$(SRCS))

ref: $(OUT)/libparref.so
ref_cuda: $(OUT)/libparref_cuda.so

$(OBJ)/%.c.o: $(REF)/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) $(call isa_of,$*.c) -c $< -o $@

$(OBJ)/%.cpp.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(call isa_of,$*.cpp) -c $< -o $@

$(OBJ)/ref_shim.o: oracle/ref_shim.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(ISA) -c $< -o $@

$(OUT)/libparref.so: $(REF_OBJS) $(OBJ)/ref_shim.o
	$(CXX) -shared -o $@ $^ -lpthread

# the PAR2ProcCUDA adapter, compiled against the reference's controller.h,
# and its test driver; linked with the CUDA backend library
$(OBJ)/controller_cuda.o: parpar_gb300/adapter/controller_cuda.cpp parpar_gb300/adapter/controller_cuda.h include/par2cuda.h
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(ISA) -I$(REF)/gf16 -Iinclude -Iparpar_gb300/adapter -c $< -o $@

$(OBJ)/adapter_shim.o: oracle/adapter_shim.cpp parpar_gb300/adapter/controller_cuda.h
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(ISA) -I$(REF)/gf16 -Iinclude -Iparpar_gb300/adapter -c $< -o $@

$(OUT)/libparref_cuda.so: $(REF_OBJS) $(OBJ)/controller_cuda.o $(OBJ)/adapter_shim.o parpar_gb300/libpar2cuda.so
	$(CXX) -shared -o $@ $(REF_OBJS) $(OBJ)/controller_cuda.o $(OBJ)/adapter_shim.o \
	    -Lparpar_gb300 -lpar2cuda -Wl,-rpath,'$$ORIGIN/../../parpar_gb300' -lpthread

clean:
	rm -rf $(OBJ) $(OUT)/libparref.so $(OUT)/libparref_cuda.so

.PHONY: ref ref_cuda clean
