# Builds the UNMODIFIED reference C backend from its own sources (read in
# place, never copied) into oracle/_ref/, the way tupan/lib/cffi_backend.py
# builds it (-O3 -std=c99, CONFIG_USE_DOUBLE for float64, libm).
# REF is the root of a reference tree (its tupan/lib/src holds the C
# sources): the installed copy baseline/_ref, or $TUPAN_REF.  Outputs are
# git-ignored.
#   make -f oracle/ref.mk REF=baseline/_ref
REF ?= $(TUPAN_REF)
ifeq ($(strip $(REF)),)
$(error set REF=<reference root> or TUPAN_REF)
endif
SRC := $(REF)/tupan/lib/src
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(HERE)_ref
FILES := phi_kernel.c acc_kernel.c acc_jerk_kernel.c snap_crackle_kernel.c \
         tstep_kernel.c pnacc_kernel.c nreg_kernels.c sakura_kernel.c \
         kepler_solver_kernel.c
SRCS := $(addprefix $(SRC)/,$(FILES))
CFLAGS = -O3 -std=c99 -fPIC -I$(SRC)

all: $(OUT)/libtupan_ref_f64.so $(OUT)/libtupan_ref_f32.so

$(OUT)/libtupan_ref_f64.so: $(SRCS)
	mkdir -p $(OUT)
	$(CC) $(CFLAGS) -DCONFIG_USE_DOUBLE=1 -shared -o $@ $(SRCS) -lm

$(OUT)/libtupan_ref_f32.so: $(SRCS)
	mkdir -p $(OUT)
	$(CC) $(CFLAGS) -shared -o $@ $(SRCS) -lm
.PHONY: all
