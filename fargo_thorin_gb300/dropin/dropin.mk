# The reference's sequential FARGO_THORIN build with the hydro loop on the GPU:
# its own src_main and src_reb sources, compiled where they lie, plus
# AlgoGasGPU.c, linked against libthorin_gpu.so.  main.c is compiled with
# -DAlgoGas=AlgoGasGPU, so its AlgoGas call (main.c:201) runs the GPU loop;
# SourceEuler.c still defines the CPU AlgoGas, which is then never called.
#
# Usage: make -f fargo_thorin_gb300/dropin/dropin.mk REF=<reference source tree> [SOREPS=1e-8]
# Output: fargo_thorin_gb300/_build/dropin/thorin_gpu (run it like the
# reference's thorin binary; it finds libthorin_gpu.so through its rpath).
ifeq ($(REF),)
  $(error REF must name the reference source tree)
endif
HERE   := $(abspath $(dir $(lastword $(MAKEFILE_LIST))))
PKG    := $(abspath $(HERE)/..)
OUT    ?= $(PKG)/_build/dropin
CC     ?= gcc
CFLAGS ?= -O3 -std=c99 -w -D_GNU_SOURCE
REBSRC := rebound.c tree.c particle.c gravity.c integrator.c integrator_whfast.c \
          integrator_whfasthelio.c integrator_ias15.c integrator_sei.c integrator_leapfrog.c \
          integrator_hermes.c boundary.c input.c output.c collision.c communication_mpi.c \
          tools.c derivatives.c simulationarchive.c
MAINSRC := LowTasks.c SideEuler.c Output.c Init.c Theo.c Interpret.c SourceEuler.c \
           TransportEuler.c Planet.c Viscosity.c Psys.c Force.c Drag.c var.c Pframeforce.c \
           split.c merge.c commbound.c fpe.c rebin.c mpiTasks.c EnergySources.c Opacity.c \
           Opacity2.c ReboundInterface.c Pebbles.c mpi_dummy.c
SORDEF := $(if $(SOREPS),-DTHORIN_DROPIN_SOREPS=$(SOREPS),)
INC    := -I$(REF)/src_main -I$(REF)/src_reb -I$(PKG)/../include

all: $(OUT)/thorin_gpu

$(OUT)/main.o: $(REF)/src_main/main.c
	mkdir -p $(OUT)
	$(CC) $(CFLAGS) $(INC) -DAlgoGas=AlgoGasGPU -c $< -o $@

$(OUT)/AlgoGasGPU.o: $(HERE)/AlgoGasGPU.c $(PKG)/../include/thorin_gpu.h $(PKG)/../include/thorin_warmnet.h
	mkdir -p $(OUT)
	$(CC) $(CFLAGS) $(INC) $(SORDEF) -c $< -o $@

$(OUT)/thorin_gpu: $(OUT)/main.o $(OUT)/AlgoGasGPU.o $(PKG)/libthorin_gpu.so \
                   $(addprefix $(REF)/src_main/,$(MAINSRC)) $(addprefix $(REF)/src_reb/,$(REBSRC))
	cd $(REF)/src_main && $(CC) $(CFLAGS) -I../src_reb $(MAINSRC) $(addprefix ../src_reb/,$(REBSRC)) \
	  $(OUT)/main.o $(OUT)/AlgoGasGPU.o -L$(PKG) -lthorin_gpu -Wl,-rpath,$(PKG) -lm -o $@
