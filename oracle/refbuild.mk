# Compiles the reference OGS-5 (test infrastructure only) straight from its
# sources with g++, in the two linear-solver configurations the oracle needs:
#
#   SP  (-DNEW_EQS): Linear_EQS / CSparseMatrix / SparseTable, the stack the
#       GPU path replaces (FEM/equation_class.cpp).
#   FEM (legacy RF): solver.cpp + matrix_routines.cpp -- SpCG, MXRandbed
#       (symmetric Dirichlet) and M34Vorkond (incomplete LDU).
#
# The source lists are those of the reference's own library definitions
# (Base, MathLib, GEO, MSH, FEM, FileIO, ThirdParty/Brent; FEM/CMakeLists.txt
# swaps equation_class.cpp for solver.cpp + matrix_routines.cpp in the legacy
# configuration). The reference's build system is not run. Its one generated
# source, Base/BuildInfo.cpp (version strings), is replaced by
# buildinfo_stub.cpp in this folder.
#
# Products, all under _ref/ (git-ignored; nothing here ships in the product):
#   _ref/libogs5_sp.a, _ref/libogs5_fem.a    the two configurations
#   _ref/ogs_sp, _ref/ogs_fem                 the reference's own main
#                                              (OGS/rf.cpp), for timing
#   _ref/ref_assemble_sp, _ref/ref_assemble_fem  ref_assemble_harness.cpp:
#       reads a deck through the reference's Problem, runs its own
#       GlobalAssembly / linear solver and writes the system in binary.
#
# Usage: make -f refbuild.mk -j8 [REF=/path/to/reference]

REF ?= /root/reference
CXX ?= g++
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref

REF_DIRS_INC := Base FEM FileIO FileIO/FEMIO FileIO/MeshIO FileIO/GeoIO FileIO/MathIO \
                GCC GEM GEO MathLib MathLib/LinAlg MSH MSHGEOTOOLS ThirdParty ThirdParty/Brent
INC := $(addprefix -I$(REF)/,$(REF_DIRS_INC))

# -ffp-contract=off: no fused multiply-adds, so both x86 and Arm hosts round as
# the reference's own x86 build without -march flags does.
CXXFLAGS_REF := -std=gnu++11 -O2 -ffp-contract=off -fPIC -w -DNDEBUG -DGCC -DHAVE_PTHREADS \
                -DHAVE_64_BIT -DIPMGEMPLUGIN -D__unix $(INC)

BASE_SRCS := $(addprefix Base/,binarySearch.cpp break.cpp DateTools.cpp display.cpp FileTools.cpp \
               makros.cpp memory.cpp MemWatch.cpp StringTools.cpp timer.cpp)
MATH_SRCS := $(addprefix MathLib/,AnalyticalGeometry.cpp EarClippingTriangulation.cpp \
               InterpolationAlgorithms/CubicSpline.cpp \
               InterpolationAlgorithms/PiecewiseLinearInterpolation.cpp LinkedTriangle.cpp MathTools.cpp)
GEO_SRCS := $(addprefix GEO/,AxisAlignedBoundingBox.cpp BruteForceClosestPair.cpp Color.cpp geo_dom.cpp \
              geo_lib.cpp geo_lin.cpp geo_mathlib.cpp geo_ply.cpp geo_pnt.cpp geo_sfc.cpp geo_vol.cpp \
              GEOObjects.cpp GeoType.cpp Point.cpp PointVec.cpp Polygon.cpp Polyline.cpp \
              PolylineWithSegmentMarker.cpp ProjectData.cpp Raster.cpp SensorData.cpp \
              SimplePolygonTree.cpp Station.cpp Surface.cpp SurfaceGrid.cpp Triangle.cpp)
MSH_SRCS := $(addprefix MSH/,GridAdapter.cpp MeshNodesAlongPolyline.cpp msh_core.cpp msh_edge.cpp \
              msh_elem.cpp msh_faces.cpp msh_lib.cpp msh_mesh.cpp msh_node.cpp MshEditor.cpp MSHEnums.cpp)
FILEIO_SRCS := $(addprefix FileIO/,FEMIO/BoundaryConditionIO.cpp FEMIO/GeoIO.cpp FEMIO/ProcessIO.cpp \
                 MeshIO/LegacyVtkInterface.cpp MeshIO/OGSMeshIO.cpp OGSIOVer4.cpp \
                 readNonBlankLineFromInputStream.cpp StationIO.cpp Writer.cpp XmlIO/RapidXMLInterface.cpp)
FEM_COMMON := $(addprefix FEM/,BoundaryCondition.cpp burgers.cpp CAP_IO.cpp conversion_rate.cpp \
                DistributionInfo.cpp DUMUX.cpp Eclipse.cpp eos.cpp fem_ele.cpp fem_ele_std.cpp \
                fem_ele_std1.cpp fem_ele_std_tes.cpp fem_ele_std_tneq.cpp fem_ele_vec.cpp \
                FEMCondition.cpp FEMEnums.cpp femlib.cpp files0.cpp GeoInfo.cpp InitialCondition.cpp \
                invariants.cpp LinearFunctionData.cpp mathlib.cpp matrix_class.cpp minkley.cpp \
                Output.cpp pcs_dm.cpp problem.cpp ProcessInfo.cpp rf_bc_new.cpp rf_fct.cpp \
                rf_fluid_momentum.cpp rf_ic_new.cpp rf_kinreact.cpp rf_mfp_new.cpp rf_mmp_new.cpp \
                rf_msp_new.cpp rf_node.cpp rf_num_new.cpp rf_out_new.cpp rf_pcs.cpp \
                rf_random_walk.cpp rf_react.cpp rf_react_cap.cpp rf_react_int.cpp rf_st_new.cpp \
                rf_tim_new.cpp rfmat_cp.cpp SourceTerm.cpp SparseMatrixDOK.cpp \
                Stiff_Bulirsch-Stoer.cpp tools.cpp vtk.cpp ShapeFunctionPool.cpp \
                Material/Fluid/GibbsFreeEnergy/DimensionLessGibbsFreeEnergyRegion1.cpp \
                Material/Fluid/Viscosity/WaterViscosityIAPWS.cpp Material/Solid/BGRaCreep.cpp par_ddc.cpp)
GCC_SRCS := $(addprefix GCC/,Density.cpp DiffOH.cpp HKF.cpp IAPWS-IF97.cpp IO.cpp logk.cpp NR.cpp \
              PITZdata.cpp VLE.cpp)
BRENT_SRCS := ThirdParty/Brent/brent.cpp

COMMON_SRCS := $(BASE_SRCS) $(MATH_SRCS) $(GEO_SRCS) $(MSH_SRCS) $(FILEIO_SRCS) $(FEM_COMMON) \
               $(GCC_SRCS) $(BRENT_SRCS)
SP_SRCS := $(COMMON_SRCS) FEM/equation_class.cpp
FEM_SRCS := $(COMMON_SRCS) FEM/solver.cpp FEM/matrix_routines.cpp

SP_OBJS := $(patsubst %.cpp,$(OUT)/sp/%.o,$(SP_SRCS)) $(OUT)/sp/buildinfo_stub.o
FEM_OBJS := $(patsubst %.cpp,$(OUT)/fem/%.o,$(FEM_SRCS)) $(OUT)/fem/buildinfo_stub.o

all: $(OUT)/ref_assemble_sp $(OUT)/ref_assemble_fem $(OUT)/ogs_sp $(OUT)/ogs_fem

$(OUT)/sp/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	@$(CXX) $(CXXFLAGS_REF) -DNEW_EQS -c -o $@ $<

$(OUT)/fem/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	@$(CXX) $(CXXFLAGS_REF) -c -o $@ $<

$(OUT)/sp/buildinfo_stub.o: $(HERE)buildinfo_stub.cpp
	@mkdir -p $(dir $@)
	@$(CXX) $(CXXFLAGS_REF) -DNEW_EQS -DOGS_STUB_SOLVER='"Alternative linear solver package (NEW_EQS)"' -c -o $@ $<

$(OUT)/fem/buildinfo_stub.o: $(HERE)buildinfo_stub.cpp
	@mkdir -p $(dir $@)
	@$(CXX) $(CXXFLAGS_REF) -DOGS_STUB_SOLVER='"Default"' -c -o $@ $<

$(OUT)/libogs5_sp.a: $(SP_OBJS)
	@rm -f $@ && ar rcs $@ $^

$(OUT)/libogs5_fem.a: $(FEM_OBJS)
	@rm -f $@ && ar rcs $@ $^

$(OUT)/ogs_sp: $(OUT)/libogs5_sp.a $(REF)/OGS/rf.cpp $(REF)/OGS/ogs_display.cpp
	@$(CXX) $(CXXFLAGS_REF) -DNEW_EQS -o $@ $(REF)/OGS/rf.cpp $(REF)/OGS/ogs_display.cpp $(OUT)/libogs5_sp.a -lpthread

$(OUT)/ogs_fem: $(OUT)/libogs5_fem.a $(REF)/OGS/rf.cpp $(REF)/OGS/ogs_display.cpp
	@$(CXX) $(CXXFLAGS_REF) -o $@ $(REF)/OGS/rf.cpp $(REF)/OGS/ogs_display.cpp $(OUT)/libogs5_fem.a -lpthread

$(OUT)/ref_assemble_sp: $(OUT)/libogs5_sp.a $(HERE)ref_assemble_harness.cpp
	@$(CXX) $(CXXFLAGS_REF) -DNEW_EQS -o $@ $(HERE)ref_assemble_harness.cpp $(OUT)/libogs5_sp.a -lpthread

$(OUT)/ref_assemble_fem: $(OUT)/libogs5_fem.a $(HERE)ref_assemble_harness.cpp
	@$(CXX) $(CXXFLAGS_REF) -o $@ $(HERE)ref_assemble_harness.cpp $(OUT)/libogs5_fem.a -lpthread

.PHONY: all
