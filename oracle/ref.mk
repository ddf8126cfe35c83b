# Build the reference (Ludwig v0.23, serial + OpenMP) from its own source
# files, in place, into oracle/_ref/.  Used only to pin the oracle and to
# generate golden fixtures; nothing shipped links against it.
#
#   make -f oracle/ref.mk REF=/root/reference -j8
#
# Flags: -O2, OpenMP, D3Q19, and -ffp-contract=off so that no multiply-add
# is fused (x86-64 baseline has no FMA; aarch64 would otherwise contract).

REF     ?= /root/reference
OUT     ?= $(dir $(lastword $(MAKEFILE_LIST)))_ref
CC      ?= gcc
CFLAGS  := -O2 -fopenmp -ffp-contract=off -DNDEBUG -D_D3Q19_ -w \
           -I$(REF)/src -I$(REF)/target -I$(REF)/mpi_s

SRCS    := $(filter-out $(REF)/src/main.c,$(wildcard $(REF)/src/*.c)) \
           $(REF)/target/target_x86.c $(REF)/mpi_s/mpi_serial.c
OBJS    := $(patsubst %.c,$(OUT)/obj/%.o,$(notdir $(SRCS)))

vpath %.c $(REF)/src $(REF)/target $(REF)/mpi_s

HERE    := $(dir $(lastword $(MAKEFILE_LIST)))

all: $(OUT)/libludwig_ref.a $(OUT)/Ludwig.exe $(OUT)/ref_shim \
     $(OUT)/length_from_sk

$(OUT)/obj/%.o: %.c
	@mkdir -p $(OUT)/obj
	$(CC) $(CFLAGS) -c $< -o $@

$(OUT)/libludwig_ref.a: $(OBJS)
	ar -crs $@ $(OBJS)

$(OUT)/Ludwig.exe: $(REF)/src/main.c $(OUT)/libludwig_ref.a
	$(CC) $(CFLAGS) $< $(OUT)/libludwig_ref.a -lm -o $@

$(OUT)/ref_shim: $(HERE)ref_shim.c $(OUT)/libludwig_ref.a
	$(CC) $(CFLAGS) $< $(OUT)/libludwig_ref.a -lm -o $@

# The reference's L(t) utility, unmodified (it reads a 128^3 binary phi
# file), against the FFTW3 interface of oracle/fftw_api (FFTW3 itself is
# not installed; the five calls it makes are implemented there).
$(OUT)/length_from_sk: $(REF)/util/length_from_sk.c $(HERE)fftw_api/fftw_dft.c \
                       $(HERE)fftw_api/fftw3.h
	@mkdir -p $(OUT)
	$(CC) -O2 -fopenmp -ffp-contract=off -w -I$(HERE)fftw_api \
	  $(REF)/util/length_from_sk.c $(HERE)fftw_api/fftw_dft.c -lm -o $@

.PHONY: all
