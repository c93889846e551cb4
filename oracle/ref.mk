# Builds programs of the reference tree, unmodified and by path, against the
# hostmpi oracle.  TEST INFRASTRUCTURE ONLY: the results pin the oracle to the
# reference's own programs and their built-in verification.  Outputs go to
# _ref/ (git-ignored).  Needs the reference tree (REF); nothing here runs on
# the GPU.
#   make -f ref.mk            cpi, NPB IS classes S, W, A and NPB DT class S
#   make -f ref.mk conv       the same programs and global_var.c passed through
#                             the source converter (_ref/conv/), so a machine
#                             without the reference tree can build them for the
#                             GPU and for hostmpi
#   make -f ref.mk if-present all and conv when the reference tree exists, else
#                             nothing (used by the build step)
#   make -s -f ref.mk print-ref   the reference tree's path (tests read it here)
# The reference tree: GPUMPI_REFERENCE_TREE when set, else its usual mount point.
REF ?= $(or $(GPUMPI_REFERENCE_TREE),/root/reference)
NPB := $(REF)/toolchain_tests/npb/NPB3.4.1/NPB3.4-MPI
O := _ref
CFLAGS := -O2 -ffp-contract=off -fno-fast-math -Ihostmpi/include -Dmain=hostmpi_user_main
LIBS := build/libhostmpi.a -lstdc++ -lpthread -lm
# NPB's print routine reports how it was built; make.def would define these
NPBDEFS := -DNPBVERSION='"3.4.1"' -DCOMPILETIME='"n/a"' -DMPICC='"gcc"' -DCFLAGS='"-O2"' \
           -DCLINK='"gcc"' -DCLINKFLAGS='""' -DCMPI_LIB='"hostmpi"' -DCMPI_INC='""'

all: $(O)/cpi $(O)/is.S $(O)/is.W $(O)/is.A $(O)/dt.S

$(O):
	mkdir -p $@

build/libhostmpi.a:
	$(MAKE) build/libhostmpi.a

$(O)/cpi: $(REF)/toolchain_tests/pi/cpi.c build/libhostmpi.a | $(O)
	gcc $(CFLAGS) $< $(LIBS) -o $@

$(O)/setparams: $(NPB)/sys/setparams.c | $(O)
	gcc -O1 $< -o $@

$(O)/is.%: $(NPB)/IS/is.c $(O)/setparams build/libhostmpi.a | $(O)
	mkdir -p $(O)/is_$*
	cd $(O)/is_$* && ../setparams is $* > /dev/null 2>&1 ; test -f npbparams.h
	gcc $(CFLAGS) $(NPBDEFS) -I$(O)/is_$* -I$(NPB)/common $< $(NPB)/common/c_print_results.c \
	    $(NPB)/common/c_timers.c $(LIBS) -o $@

$(O)/dt.%: $(NPB)/DT/dt.c $(NPB)/DT/DGraph.c $(O)/setparams build/libhostmpi.a | $(O)
	mkdir -p $(O)/dt_$*
	cd $(O)/dt_$* && ../setparams dt $* > /dev/null 2>&1 ; test -f npbparams.h
	gcc $(CFLAGS) $(NPBDEFS) -I$(O)/dt_$* -I$(NPB)/common $(NPB)/DT/dt.c $(NPB)/DT/DGraph.c \
	    $(NPB)/common/c_print_results.c $(NPB)/common/c_timers.c $(NPB)/common/randdp.c $(LIBS) -o $@

CONV := python3 ../dphpc-project_gb300/gpumpi_convert.py
C := $(O)/conv
conv: $(C)/cpi/cpi.cu $(C)/global_var/global_var.cu $(C)/is_S/npbparams.h.cuh \
      $(C)/is_W/npbparams.h.cuh $(C)/is_A/npbparams.h.cuh $(C)/dt_S/npbparams.h.cuh

$(C)/cpi/cpi.cu: $(REF)/toolchain_tests/pi/cpi.c ../dphpc-project_gb300/gpumpi_convert.py
	$(CONV) $< --project $(REF)/toolchain_tests/pi --outdir $(C)/cpi

$(C)/global_var/global_var.cu: $(REF)/toolchain_tests/global_var/global_var.c ../dphpc-project_gb300/gpumpi_convert.py
	$(CONV) $< --project $(REF)/toolchain_tests/global_var --outdir $(C)/global_var

# npbparams.h per class beside its converted .cuh; the converted IS sources do
# not depend on the class (it is read from npbparams.h at compile time)
$(C)/is_%/npbparams.h.cuh: $(NPB)/IS/is.c $(O)/setparams ../dphpc-project_gb300/gpumpi_convert.py
	mkdir -p $(C)/is_$*
	cd $(C)/is_$* && ../../setparams is $* > /dev/null 2>&1 ; test -f npbparams.h
	for f in IS/is.c common/c_print_results.c common/c_timers.c; do \
	    $(CONV) $(NPB)/$$f --project $(NPB) -I $(C)/is_$* --outdir $(C)/npb || exit 1; done

$(C)/dt_%/npbparams.h.cuh: $(NPB)/DT/dt.c $(O)/setparams ../dphpc-project_gb300/gpumpi_convert.py
	mkdir -p $(C)/dt_$*
	cd $(C)/dt_$* && ../../setparams dt $* > /dev/null 2>&1 ; test -f npbparams.h
	for f in DT/dt.c DT/DGraph.c common/randdp.c common/c_print_results.c common/c_timers.c; do \
	    $(CONV) $(NPB)/$$f --project $(NPB) -I $(C)/dt_$* --outdir $(C)/npb || exit 1; done

print-ref:
	@echo $(REF)

if-present:
	@if [ -d "$(REF)/toolchain_tests" ]; then $(MAKE) -f ref.mk all conv; \
	 else echo "reference tree not found at $(REF): _ref/ not built"; fi

.PHONY: all conv print-ref if-present
