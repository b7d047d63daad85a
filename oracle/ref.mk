# Builds the reference-code oracle: the reference's own headers, unmodified,
# compiled from where they lie against this project's ParlayLib-API stand-in
# (oracle/ref_shim/), with C entry points (oracle/ref_bridge_*.cpp).
# Outputs go to oracle/_ref/ only.  Test infrastructure: the product never
# links these libraries.
#
#   make -f oracle/ref.mk REF=/root/reference        (from the repository root)
#
# The reference's own Makefile (src/Makefile) is not used: it needs the
# absent ParlayLib and adds -mcx16 -march=native -Werror.
REF ?= /root/reference
OUT := oracle/_ref
CXX ?= g++
CXXFLAGS := -std=c++17 -O2 -fopenmp -fPIC -shared -w \
            -Ioracle/ref_shim -I$(REF)/src -I$(REF)/baselines/tarjan_scc -Ioracle

LIBS := $(OUT)/libref_scc.so $(OUT)/libref_cc.so $(OUT)/libref_lelist.so
SHIM := oracle/ref_shim/psc_parlay_shim.h oracle/ref_bridge_common.hpp \
        parallel-strong-connectivity_gb300/csrc/psc_hash.h

all: $(LIBS)

$(OUT)/libref_scc.so: oracle/ref_bridge_scc.cpp $(SHIM) | $(OUT)
	$(CXX) $(CXXFLAGS) $< -o $@

$(OUT)/libref_cc.so: oracle/ref_bridge_cc.cpp $(SHIM) | $(OUT)
	$(CXX) $(CXXFLAGS) $< -o $@

$(OUT)/libref_lelist.so: oracle/ref_bridge_lelist.cpp $(SHIM) | $(OUT)
	$(CXX) $(CXXFLAGS) $< -o $@

$(OUT):
	mkdir -p $(OUT)

.PHONY: all
