# Builds oracle/_ref/libcmcref.so: the reference's own Henon-step TUs,
# compiled unmodified where they lie, against the single-rank MPI / GSL /
# HDF5 shims in oracle/refshim, with the draw sites routed to the counter
# generator the kernels use (TEST INFRASTRUCTURE; nothing in the product
# links it).  The reference's CMake build is not used: it needs MPI, GSL,
# HDF5, zlib-linked I/O and gfortran/COSMIC, none of which this image has.
#
#   make -f oracle/ref.mk [REFERENCE_ROOT=<reference tree>]
#
# Also builds oracle/_ref/libtaus113ref.so, the reference's taus113-v2.c
# alone, which pins the oracle's own taus113 generator.
#
# Flags follow the reference's CMakeLists.txt:75,86 (-DEXPERIMENTAL,
# -fcommon); -ffp-contract=off keeps a*b+c as two roundings on every host.

REFERENCE_ROOT ?= /root/reference
HERE := $(patsubst %/,%,$(dir $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)/_ref
OBJ := $(OUT)/obj
SHIM := $(HERE)/refshim
LIB := $(OUT)/libcmcref.so

CC ?= gcc
CFLAGS := -O2 -fPIC -std=gnu11 -fcommon -DEXPERIMENTAL -ffp-contract=off -fno-fast-math -w \
          -I$(SHIM) -I$(REFERENCE_ROOT)/include/cmc -I$(REFERENCE_ROOT)/include/common \
          -I$(REFERENCE_ROOT)/include
INJECT := -include $(SHIM)/cmcref_inject.h -Dexit=cmcref_exit

SRC := $(REFERENCE_ROOT)/src/cmc
# TU number and the star index / trial counter in scope at its draw sites
DRAW_cmc_dynamics := 1,__LINE__,(long)(k),0L
DRAW_cmc_dynamics_helper := 2,__LINE__,(long)(k),0L
DRAW_cmc_evolution_thr := 3,__LINE__,(long)(j),(long)(k)
DRAW_cmc_utils := 9,__LINE__,-1L,0L
DRAW_cmc_orbit := 9,__LINE__,-1L,0L
DRAW_cmc_nr := 9,__LINE__,-1L,0L
DRAW_cmc_sort := 9,__LINE__,-1L,0L
DRAW_cmc_fits := 9,__LINE__,-1L,0L
DRAW_cmc_mpi := 9,__LINE__,-1L,0L
DRAW_fewbody_utils := 9,__LINE__,-1L,0L

TUS := cmc_utils cmc_dynamics cmc_dynamics_helper cmc_evolution_thr cmc_orbit cmc_nr cmc_sort cmc_fits cmc_mpi
REF_OBJS := $(TUS:%=$(OBJ)/%.o) $(OBJ)/fewbody_utils.o $(OBJ)/taus113-v2.o
SHIM_OBJS := $(OBJ)/refshim.o $(OBJ)/refdrive.o $(OBJ)/refstubs.o

TAUS_LIB := $(OUT)/libtaus113ref.so

all: $(LIB) $(TAUS_LIB)

# the reference's generator alone, for the oracle's taus113 pin
$(TAUS_LIB): $(REFERENCE_ROOT)/src/libs/taus113-v2.c
	mkdir -p $(OUT)
	$(CC) -O2 -fPIC -shared -I$(REFERENCE_ROOT)/include/common -o $@ $<

print-root:
	@echo $(REFERENCE_ROOT)

$(OBJ):
	mkdir -p $(OBJ)

$(OBJ)/%.o: $(SRC)/%.c $(SHIM)/cmcref_inject.h $(wildcard $(SHIM)/*.h $(SHIM)/gsl/*.h) | $(OBJ)
	$(CC) $(CFLAGS) $(INJECT) '-DCMCREF_DRAW_ARGS=$(DRAW_$*)' -c $< -o $@

# Fewbody's vector helpers (fb_sqr, fb_cub, ...), which cmc_utils.c and
# cmc_evolution_thr.c call on the step
$(OBJ)/fewbody_utils.o: $(REFERENCE_ROOT)/src/fewbody-0.24/fewbody_utils.c $(SHIM)/cmcref_inject.h | $(OBJ)
	$(CC) $(CFLAGS) -I$(REFERENCE_ROOT)/include/fewbody-0.24 $(INJECT) '-DCMCREF_DRAW_ARGS=$(DRAW_fewbody_utils)' -c $< -o $@

$(OBJ)/taus113-v2.o: $(REFERENCE_ROOT)/src/libs/taus113-v2.c | $(OBJ)
	$(CC) $(CFLAGS) -c $< -o $@

$(OBJ)/refshim.o: $(SHIM)/refshim.c $(HERE)/brent1973.h $(wildcard $(SHIM)/*.h $(SHIM)/gsl/*.h) | $(OBJ)
	$(CC) $(CFLAGS) -c $< -o $@

$(OBJ)/refdrive.o: $(SHIM)/refdrive.c $(HERE)/philox.h $(wildcard $(SHIM)/*.h $(SHIM)/gsl/*.h) | $(OBJ)
	$(CC) $(CFLAGS) -c $< -o $@

$(OBJ)/refstubs.o: $(SHIM)/refstubs.c | $(OBJ)
	$(CC) $(CFLAGS) -c $< -o $@

$(LIB): $(REF_OBJS) $(SHIM_OBJS)
	$(CC) -shared -o $@ $^ -lm -Wl,--no-undefined -lz

clean:
	rm -rf $(OUT)/obj $(LIB) $(TAUS_LIB)

.PHONY: all clean print-root
