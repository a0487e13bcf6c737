# Builds the reference FARGO_THORIN binary straight from its sources (no use
# of the reference's own build system) into oracle/_ref/.
# Usage: make -f oracle/ref.mk REF=<reference source tree> [OMP=1] [SOREPS=1e-8]
# The REBOUND OpenGL viewer (display.c, glad.c) is compiled out in the
# reference (OPENGL is empty) and is left out here.
ifeq ($(REF),)
  $(error REF must name the reference source tree)
endif
OUT    ?= $(dir $(lastword $(MAKEFILE_LIST)))_ref
CC     ?= gcc
# -std=c99 keeps gcc from contracting a*b+c into FMAs, as the reference build does.
CFLAGS ?= -O3 -std=c99 -w -D_GNU_SOURCE
REBSRC := rebound.c tree.c particle.c gravity.c integrator.c integrator_whfast.c \
          integrator_whfasthelio.c integrator_ias15.c integrator_sei.c integrator_leapfrog.c \
          integrator_hermes.c boundary.c input.c output.c collision.c communication_mpi.c \
          tools.c derivatives.c simulationarchive.c
MAINSRC := LowTasks.c SideEuler.c Output.c Init.c main.c Theo.c Interpret.c SourceEuler.c \
           TransportEuler.c Planet.c Viscosity.c Psys.c Force.c Drag.c var.c Pframeforce.c \
           split.c merge.c commbound.c fpe.c rebin.c mpiTasks.c EnergySources.c Opacity.c \
           Opacity2.c ReboundInterface.c Pebbles.c
ifeq ($(OMP),1)
  SUFFIX := _omp
  XFLAGS := -fopenmp -DOPENMP
else
  SUFFIX :=
  XFLAGS := mpi_dummy.c
endif
# SOREPS, the SOR tolerance, is a #define in EnergySources.c (line 23).  A
# variant with another tolerance compiles that one file from a stream edit of
# the source (sed to the compiler's standard input, no copy on disk) and the
# rest unchanged.
ifneq ($(SOREPS),)
  SUFFIX := $(SUFFIX)_soreps$(SOREPS)
  SORMAIN := $(filter-out EnergySources.c,$(MAINSRC))
  SOROBJ := $(abspath $(OUT))/EnergySources_soreps$(SOREPS)$(if $(filter 1,$(OMP)),_omp,).o
else
  SORMAIN := $(MAINSRC)
  SOROBJ :=
endif

all: $(OUT)/thorin$(SUFFIX)

ifneq ($(SOREPS),)
$(SOROBJ): $(REF)/src_main/EnergySources.c
	mkdir -p $(OUT)
	sed 's/^#define SOREPS .*/#define SOREPS $(SOREPS)/' $< | \
	  $(CC) $(CFLAGS) $(if $(filter 1,$(OMP)),-fopenmp -DOPENMP,) -I$(REF)/src_main -I$(REF)/src_reb -x c -c - -o $@
endif

$(OUT)/thorin$(SUFFIX): $(addprefix $(REF)/src_main/,$(MAINSRC)) $(addprefix $(REF)/src_reb/,$(REBSRC)) $(SOROBJ)
	mkdir -p $(OUT)
	cd $(REF)/src_main && $(CC) $(CFLAGS) -I../src_reb $(SORMAIN) $(SOROBJ) $(XFLAGS) \
	  $(addprefix ../src_reb/,$(REBSRC)) -o $(abspath $@) -lm
