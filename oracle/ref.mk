# Builds programs of the reference tree, unmodified and by path, against the
# hostmpi oracle.  TEST INFRASTRUCTURE ONLY: the results pin the oracle to the
# reference's own programs and their built-in verification.  Outputs go to
# _ref/ (git-ignored).  Needs the reference tree (REF); nothing here runs on
# the GPU.
#   make -f ref.mk            cpi and NPB IS classes S, W, A
REF ?= /root/reference
NPB := $(REF)/toolchain_tests/npb/NPB3.4.1/NPB3.4-MPI
O := _ref
CFLAGS := -O2 -ffp-contract=off -fno-fast-math -Ihostmpi/include -Dmain=hostmpi_user_main
LIBS := build/libhostmpi.a -lstdc++ -lpthread -lm
# NPB's print routine reports how it was built; make.def would define these
NPBDEFS := -DNPBVERSION='"3.4.1"' -DCOMPILETIME='"n/a"' -DMPICC='"gcc"' -DCFLAGS='"-O2"' \
           -DCLINK='"gcc"' -DCLINKFLAGS='""' -DCMPI_LIB='"hostmpi"' -DCMPI_INC='""'

all: $(O)/cpi $(O)/is.S $(O)/is.W $(O)/is.A

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

.PHONY: all
