# Builds the reference ParaFROST CPU solver (the SIGmA simplifier lives in it)
# straight from its sources under REFDIR with g++, without the reference's own
# installer. Outputs go only to oracle/_ref/. Test infrastructure, never shipped.
#
#   make -f oracle/ref.mk REFDIR=/path/to/ParaFROST -j8
ifndef REFDIR
$(error REFDIR=<path of the ParaFROST sources> is required)
endif
OUT    := oracle/_ref
SRCDIR := $(REFDIR)/src/cpu
CXX    ?= g++
# Same optimisation flags as the reference installer's release mode, plus the two
# -include flags that g++ 13 needs because the sources rely on transitive includes.
CXXFLAGS := -std=c++17 -DNDEBUG -O3 -fPIC -w -include cstdint -include cstddef -Ioracle
SRCS := $(filter-out $(SRCDIR)/main.cpp,$(sort $(wildcard $(SRCDIR)/*.cpp)))
OBJS := $(patsubst $(SRCDIR)/%.cpp,$(OUT)/obj/%.o,$(SRCS))

all: $(OUT)/libpfref.a $(OUT)/sigma_ref $(OUT)/parafrost

$(OUT)/obj/%.o: $(SRCDIR)/%.cpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -I$(SRCDIR) -c $< -o $@

$(OUT)/libpfref.a: $(OBJS)
	ar rcs $@ $^

$(OUT)/sigma_ref: oracle/ref_harness.cpp $(OUT)/libpfref.a
	$(CXX) $(CXXFLAGS) -I$(SRCDIR) $< -o $@ $(OUT)/libpfref.a

# the reference solver's own command line (CDCL search; equisatisfiability checks)
$(OUT)/parafrost: $(SRCDIR)/main.cpp $(OUT)/libpfref.a
	$(CXX) $(CXXFLAGS) -I$(SRCDIR) $< -o $@ $(OUT)/libpfref.a

# the reference solver with its preprocessing round handed to this repository's C ABI
# (oracle/dropin_harness.cpp), linked to the kernel-logic emulation build
EMU := parafrost_gb300/_lib/libsigma_emu.so
dropin: $(OUT)/sigma_dropin
$(OUT)/sigma_dropin: oracle/dropin_harness.cpp include/sigma_gb300.hpp include/sigma_gb300.h $(OUT)/libpfref.a $(EMU)
	$(CXX) $(CXXFLAGS) -I$(SRCDIR) -Iinclude $< -o $@ $(OUT)/libpfref.a $(abspath $(EMU)) -Wl,-rpath,$(abspath $(dir $(EMU)))

.PHONY: all dropin
