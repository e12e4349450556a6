# Builds the reference's own CPU implementation of the recovery path (ParPar
# gf16/ + hasher/ cores, non-libuv std::future mode) straight from the
# reference source tree, plus oracle/ref_shim.cpp, into oracle/_ref/libparref.so.
# Test infrastructure only (pins the oracle and generates golden fixtures); it
# only builds where the reference tree exists.  Nothing is copied out of it.
#
#   make -f oracle/ref.mk REF=/root/reference
REF ?= /root/reference
OUT := oracle/_ref
OBJ := $(OUT)/obj

ARCH := $(shell uname -m)
ifeq ($(ARCH),x86_64)
# per-file ISA flags are selected at run time by the reference's CPUID dispatch;
# compiling everything for the build host enables every x86 kernel it has
ISA := -march=native
else
ISA := -march=armv8-a+crc
endif

COMMON := -O2 -DNDEBUG -fno-strict-aliasing -fPIC -I$(REF) $(ISA) -Wno-unused-function -w
CFLAGS := $(COMMON) -std=gnu99
CXXFLAGS := $(COMMON) -std=c++11 -fexceptions

GF_C := $(filter-out %opencl-include/cl.c,$(wildcard $(REF)/gf16/*.c))
GF_CXX := $(REF)/gf16/gf16mul.cpp $(REF)/gf16/controller.cpp $(REF)/gf16/controller_cpu.cpp
HS_CXX := $(wildcard $(REF)/hasher/*.cpp)
HS_C := $(REF)/hasher/crc_zeropad.c $(REF)/hasher/md5-final.c

SRCS := $(GF_C) $(GF_CXX) $(HS_CXX) $(HS_C)
OBJS := $(patsubst $(REF)/%,$(OBJ)/%.o,$(SRCS)) $(OBJ)/ref_shim.o

all: $(OUT)/libparref.so

$(OBJ)/%.c.o: $(REF)/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) -c $< -o $@

$(OBJ)/%.cpp.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/ref_shim.o: oracle/ref_shim.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libparref.so: $(OBJS)
	$(CXX) -shared -o $@ $(OBJS) -lpthread

clean:
	rm -rf $(OUT)

.PHONY: all clean
