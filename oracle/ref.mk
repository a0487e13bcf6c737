# Builds the reference FARGO_THORIN sequential binary straight from its sources
# (no use of the reference's own build system) into oracle/_ref/.
# Usage: make -f oracle/ref.mk REF=/path/to/reference [OMP=1]
# The REBOUND OpenGL viewer (display.c, glad.c) is compiled out in the
# reference (OPENGL is empty) and is left out here.
REF    ?= /root/reference
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
# SOREPS is hard-coded in EnergySources.c; SOREPS_OVERRIDE builds a variant
# with another tolerance by pre-defining it through a forced include.
ifneq ($(SOREPS),)
  SUFFIX := $(SUFFIX)_soreps$(SOREPS)
  SORDEF := -include $(OUT)/soreps$(SOREPS).h
endif

all: $(OUT)/thorin$(SUFFIX)

$(OUT)/thorin$(SUFFIX): $(addprefix $(REF)/src_main/,$(MAINSRC)) $(addprefix $(REF)/src_reb/,$(REBSRC))
	mkdir -p $(OUT)
	cd $(REF)/src_main && $(CC) $(CFLAGS) $(SORDEF) -I../src_reb $(MAINSRC) $(XFLAGS) \
	  $(addprefix ../src_reb/,$(REBSRC)) -o $(abspath $@) -lm
