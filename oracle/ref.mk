# Builds the reference's own per-cell numerics into one shared library per
# case plugin, as the checker of the oracle restatement (test infrastructure
# only; nothing in the product links these).
#
#   make -f ref.mk [REF=<reference checkout>]
#
# Each library compiles, unmodified and from where they lie in the reference
# checkout, Source/Src_3d/{compute_flux_3d,flux_schemes,consprim_funcs,div_3d,
# ib_utils}.H (through ref_driver.cpp), Source/{globalDefines,mflo_constants}.H
# and the case directory's species.H/.cpp, thermo.H, transport.H,
# userfuncs.H/.cpp and chemistry.H, against the AMReX stand-in in ref_shim/.
# Same floating-point flags as the strict oracle build.  Outputs go to _ref/
# only.
REF      ?= /root/reference
CXX      ?= g++
FLAGS    := -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w
OUT      := _ref

# name:case directory (relative to REF)
CASES := \
  stube:tests/Cartesian/ShockTube_N2 \
  stubehe:tests/Cartesian/ShockTube_N2He \
  tg:tests/Cartesian/TaylorGreen \
  speq:tests/Cartesian/SpeciesEqTests \
  porous:models/porousParticle \
  catcyl:models/catalystCylinder \
  bcat:models/blockCatalyst1d \
  stag:models/stagFlowCatalyst \
  cht:models/conjHtransferTest \
  rxn:py_utils/rxnscheme_writer/example

name_of = $(word 1,$(subst :, ,$(1)))
dir_of  = $(word 2,$(subst :, ,$(1)))
LIBS    := $(foreach c,$(CASES),$(OUT)/libref_$(call name_of,$(c)).so)
# counting builds (Real = a double that counts FP64 operations, ref_shim/count_double.H)
COUNTED := porous tg catcyl
CLIBS   := $(foreach c,$(filter $(addsuffix :%,$(COUNTED)),$(CASES)),$(OUT)/libref_count_$(call name_of,$(c)).so)

all: $(LIBS) $(CLIBS)

define case_rule
$(OUT)/libref_$(call name_of,$(1)).so: ref_driver.cpp $(wildcard ref_shim/*.H) ../include/mflo_gpu.h
	@mkdir -p $(OUT)
	$(CXX) $(FLAGS) -Iref_shim -I$(REF)/$(call dir_of,$(1)) -I$(REF)/Source -I$(REF)/Source/Src_3d -I../include \
	    -o $$@ ref_driver.cpp $(REF)/$(call dir_of,$(1))/species.cpp $(REF)/$(call dir_of,$(1))/userfuncs.cpp
$(OUT)/libref_count_$(call name_of,$(1)).so: ref_driver.cpp $(wildcard ref_shim/*.H) ../include/mflo_gpu.h
	@mkdir -p $(OUT)
	$(CXX) $(FLAGS) -DMFG_COUNT_FLOPS -Iref_shim -I$(REF)/$(call dir_of,$(1)) -I$(REF)/Source -I$(REF)/Source/Src_3d \
	    -I../include -o $$@ ref_driver.cpp $(REF)/$(call dir_of,$(1))/species.cpp $(REF)/$(call dir_of,$(1))/userfuncs.cpp
endef
$(foreach c,$(CASES),$(eval $(call case_rule,$(c))))

clean:
	rm -rf $(OUT)

.PHONY: all clean
