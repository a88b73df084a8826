// Version strings for the reference OGS-5 build made by refbuild.mk.
//
// The reference generates this translation unit at configure time from its
// own template; the oracle build does not run that step, so these constants
// (the names come from the reference's Base/BuildInfo.h) say what built it.
// Test infrastructure only.
#include "BuildInfo.h"

#ifndef OGS_STUB_SOLVER
#define OGS_STUB_SOLVER "Default"
#endif

namespace BuildInfo
{
const std::string GIT_COMMIT_INFO("unknown");
const std::string GIT_BRANCH_INFO("unknown");
const std::string BUILD_TIMESTAMP("unknown");
const std::string CMAKE_SYSTEM("linux");
const std::string CMAKE_SYSTEM_PROCESSOR("unknown");
const std::string CMAKE_CXX_COMPILER("g++");
const std::string GCC_VERSION("unknown");
const std::string CMAKE_GENERATOR("oracle/refbuild.mk");
const std::string CMAKE_BUILD_TYPE("Release");
const std::string CMAKE_CXX_FLAGS("-O2 -ffp-contract=off");
const std::string CMAKE_CXX_FLAGS_RELEASE("");
const std::string CMAKE_CXX_FLAGS_DEBUG("");
const std::string SOLVER_PACKAGE_NAME(OGS_STUB_SOLVER);
const std::string SOURCEPATH("");
const std::string BUILDPATH("");
const std::string TESTDATAPATH("");
const std::string OGS_VERSION("5 (oracle build)");
const std::string OGS_DATE("");
const std::string OGS_EXECUTABLE("ogs");
const std::string PUT_TMP_DIR_IN("");
}  // namespace BuildInfo
