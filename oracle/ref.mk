# Test infrastructure only: builds the UNMODIFIED CPU path of the reference
# (moarseniy/CudaFEMproject, FEMproject/) straight from its sources with g++,
# linked to the project-owned driver oracle/ref_driver.cpp. Nothing here is
# shipped or measured as the product; the binary is used by tests (FP32 cross
# check of the oracle) and as the CPU baseline where it can be built.
#
#   make -f oracle/ref.mk REF=<reference checkout>/FEMproject
#   (or CFEM_REFERENCE_ROOT=<reference checkout> make -f oracle/ref.mk)
#
# Outputs go to oracle/_ref/ only (git-ignored). The reference's own CMake
# build is not used; its CUDA backend is left out (WITH_CUDA undefined), which
# is exactly the DEVICE_NAME == CPU path of femfunc.cpp.

REF ?= $(CFEM_REFERENCE_ROOT)/FEMproject
OUT ?= oracle/_ref
CXX ?= g++
# -ffp-contract=off: no FMA contraction, so x86 and aarch64 round alike.
CXXFLAGS ?= -O3 -DNDEBUG -std=c++17 -ffp-contract=off -w

INC = -I$(REF)/matrix_pack/include -I$(REF)/fem_utils/include \
      -I$(REF)/DataKeeper/src -I$(REF)/femstruct/src -I$(REF)/Tools/src \
      -I$(REF)/VTKfile/src -I$(REF)/femfunc/src \
      -I$(REF)/thirdparty/segyio/include -I$(REF)/thirdparty/json/single_include \
      -I$(REF)/thirdparty -I$(REF)/thirdparty/segyio2/include -I$(REF)/segyUtils/src

SRCS = $(REF)/femfunc/src/femfunc.cpp \
       $(REF)/fem_utils/src/fem_utils.cpp \
       $(REF)/fem_utils/src/cpu_fem_utils.cpp \
       $(REF)/matrix_pack/src/matrix_pack.cpp \
       $(REF)/matrix_pack/src/cpu_matrix.cpp \
       $(REF)/DataKeeper/src/datakeeper.cpp \
       $(REF)/femstruct/src/femstruct.cpp \
       $(REF)/Tools/src/Tools.cpp \
       $(REF)/VTKfile/src/VTKfile.cpp \
       $(REF)/thirdparty/segyio/src/SegyIO.cpp \
       $(REF)/thirdparty/segyio/src/SegyIn.cpp \
       $(REF)/thirdparty/segyio/src/SegyOut.cpp \
       $(REF)/segyUtils/src/segyUtils.cpp
CSRCS = $(REF)/thirdparty/segyio2/src/segy.c
CC ?= gcc

OBJS = $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(SRCS)) $(patsubst $(REF)/%.c,$(OUT)/obj/%.c.o,$(CSRCS))

all: $(OUT)/ref_driver

$(OUT)/obj/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/obj/%.c.o: $(REF)/%.c
	@mkdir -p $(dir $@)
	$(CC) -O2 -std=gnu99 -w $(INC) -c $< -o $@

$(OUT)/obj/ref_driver.o: oracle/ref_driver.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/ref_driver: $(OBJS) $(OUT)/obj/ref_driver.o
	$(CXX) -o $@ $(OUT)/obj/ref_driver.o -Wl,--start-group $(OBJS) -Wl,--end-group

# the include list and the reference's objects, for callers that compile and
# link their own code against the reference (tests/test_integration_branch.py)
print-inc:
	@echo $(INC)

print-objs:
	@echo $(OBJS)

objs: $(OBJS)

clean:
	rm -rf $(OUT)

.PHONY: all clean print-inc print-objs objs
