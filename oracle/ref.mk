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

all: $(OUT)/libludwig_ref.a $(OUT)/Ludwig.exe $(OUT)/ref_shim

$(OUT)/obj/%.o: %.c
	@mkdir -p $(OUT)/obj
	$(CC) $(CFLAGS) -c $< -o $@

$(OUT)/libludwig_ref.a: $(OBJS)
	ar -crs $@ $(OBJS)

$(OUT)/Ludwig.exe: $(REF)/src/main.c $(OUT)/libludwig_ref.a
	$(CC) $(CFLAGS) $< $(OUT)/libludwig_ref.a -lm -o $@

$(OUT)/ref_shim: $(dir $(lastword $(MAKEFILE_LIST)))ref_shim.c $(OUT)/libludwig_ref.a
	$(CC) $(CFLAGS) $< $(OUT)/libludwig_ref.a -lm -o $@

.PHONY: all
