# Builds the reference Radiance programs that pin the oracle: rtrace, rcontrib,
# oconv, obj2mesh, dctimestep, rfluxmtx and rmtxop, compiled straight from the reference's own C sources
# (read in place, never copied) with the reference's release flags.
#
#   make -f oracle/build_ref.mk REF=/root/reference -j8
#
# Outputs go to oracle/_ref/ only (git-ignored). The programs are test
# infrastructure: they generate golden vectors for tests/golden and may be
# timed as the CPU baseline where the reference tree is present.
REF     ?= /root/reference
RAD     := $(REF)/src/radiance
OUT     := oracle/_ref
OBJ     := $(OUT)/obj
CC      ?= gcc
CXX     ?= g++
CFLAGS  := -O3 -ffast-math -funroll-loops -w -Dlinux -D_FILE_OFFSET_BITS=64 \
           -DNOSTEREO -Derror=rad_error -I$(RAD)/common -I$(RAD)/rt

COMMON_C := cone face instance readobj readoct otypes objset octree readfargs \
  modobject getlibpath zeroes mesh readmesh tmesh sceneio free_os addobjnotify \
  color header image lamps resolu rexpr spec_rgb colrops font tonemap tmapcolrs \
  tmapluv tmap16bit bmpfile falsecolor depthcodec normcodec idmap fltdepth \
  jitteraperture ezxml ccolor ccyrgb bsdf bsdf_m bsdf_t loadbsdf disk2square \
  hilbert interp2d triangulate data fgetline fropen linregr xf mat4 invmat4 \
  fvect urand urind calexpr caldefn calfunc calprnt biggerlib multisamp process \
  gethomedir getpath error savestr savqstr badarg fgetword words expandarg \
  wordfile fgetval clip plocate eputs wputs quit lookup bmalloc tcos fputword \
  dircode paths byteswap cvtcmd dmessage fixargv0 chanvalue loadvars \
  unix_process ealloc fdate portio myhostname erf strnstr strlcpy
COMMON_CXX := abitmap abitmapio
RT_C := ambcomp ambient ambio freeobjmem initotypes preload raytrace renderopts \
  source sphere srcobstr srcsupp srcsamp virtuals o_face o_cone o_instance \
  o_mesh aniso normal dielectric m_clip glass m_brdf m_mirror m_direct m_mist \
  m_wgmdf fprism m_alias m_bsdf ashikhmin p_func t_func p_data t_data text \
  mx_func mx_data func noise3 pmap pmapsrc pmapmat pmaprand pmapio pmapdata \
  pmapbias pmapparm pmapcontrib pmapamb pmapray pmapopt pmapdiag pmaptype \
  oocmorton oococt oocsort oocbuild oocnn ooccache pmutil pmcontrib2 Version
RL_C := raycalls rayfifo raypcalls

COMMON_O := $(addprefix $(OBJ)/common/,$(addsuffix .o,$(COMMON_C) $(COMMON_CXX)))
RT_O := $(addprefix $(OBJ)/rt/,$(addsuffix .o,$(RT_C)))
RL_O := $(addprefix $(OBJ)/rt/,$(addsuffix .o,$(RL_C)))

LIBRTRAD := $(OBJ)/librtrad.a
LIBRAD   := $(OBJ)/libradiance.a
LIBRL    := $(OBJ)/libraycalls.a

CALS := $(RAD)/rt/rayinit.cal $(RAD)/util/reinhartb.cal $(RAD)/util/klems_full.cal $(RAD)/util/klems_half.cal \
        $(RAD)/util/klems_quarter.cal $(RAD)/util/disk2square.cal $(RAD)/util/cieskyscan.cal

all: $(OUT)/bin/rtrace $(OUT)/bin/rcontrib $(OUT)/bin/oconv $(OUT)/bin/obj2mesh $(OUT)/bin/dctimestep $(OUT)/bin/rfluxmtx $(OUT)/bin/rmtxop
	@mkdir -p $(OUT)/lib && cp $(CALS) $(OUT)/lib/

$(OBJ)/common/%.o: $(RAD)/common/%.c
	@mkdir -p $(@D)
	$(CC) $(CFLAGS) -c $< -o $@
$(OBJ)/common/%.o: $(RAD)/common/%.cpp
	@mkdir -p $(@D)
	$(CXX) $(CFLAGS) -c $< -o $@
$(OBJ)/rt/%.o: $(RAD)/rt/%.c
	@mkdir -p $(@D)
	$(CC) $(CFLAGS) -c $< -o $@
$(OBJ)/ot/%.o: $(RAD)/ot/%.c
	@mkdir -p $(@D)
	$(CC) $(CFLAGS) -I$(RAD)/ot -c $< -o $@
$(OBJ)/util/%.o: $(RAD)/util/%.c
	@mkdir -p $(@D)
	$(CC) $(CFLAGS) -I$(RAD)/util -c $< -o $@

$(LIBRTRAD): $(COMMON_O)
	rm -f $@ && ar rcs $@ $^
$(LIBRAD): $(RT_O)
	rm -f $@ && ar rcs $@ $^
$(LIBRL): $(RL_O)
	rm -f $@ && ar rcs $@ $^

$(OUT)/bin/rtrace: $(addprefix $(OBJ)/rt/,rtmain.o rtrace.o duphead.o persist.o) $(LIBRL) $(LIBRAD) $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm
$(OUT)/bin/rcontrib: $(addprefix $(OBJ)/rt/,rcmain.o rcontrib.o rc2.o rc3.o) $(LIBRAD) $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm
$(OUT)/bin/oconv: $(addprefix $(OBJ)/ot/,bbox.o initotypes.o o_cone.o o_face.o o_instance.o oconv.o sphere.o writeoct.o) $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm
$(OUT)/bin/obj2mesh: $(addprefix $(OBJ)/ot/,cvmesh.o o_face.o obj2mesh.o wfconv.o writemesh.o) $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm
$(OUT)/bin/rmtxop: $(addprefix $(OBJ)/util/,rmtxop.o rmatrix.o cmconst.o cmbsdf.o cmatrix.o rmconvert.o) $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm
$(OUT)/bin/rfluxmtx: $(OBJ)/util/rfluxmtx.o $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm
$(OUT)/bin/dctimestep: $(addprefix $(OBJ)/util/,dctimestep.o cmbsdf.o cmconst.o cmatrix.o) $(LIBRTRAD)
	@mkdir -p $(@D)
	$(CXX) -o $@ $^ -lm

.PHONY: all
