// Definitions of the reference's config.h globals for the oracle reference
// build.  The reference hard-codes them in config.cpp; here each one is read
// once, at load time, from an environment variable (KF_REF_<NAME>), so that a
// test can load a private copy of the library per parameter set.  The solver
// is put in its race-free Jacobi schedule (UpdateAllVoxelsInEachIter and
// UsePreviousIterationDeformationField, KillingFusion.cpp:248-352).
// TEST INFRASTRUCTURE ONLY.
#include <cstdlib>
#include <string>

#include <config.h>

static double envd(const char *name, double dflt) {
  const char *v = std::getenv(name);
  return v ? std::strtod(v, nullptr) : dflt;
}
static int envi(const char *name, int dflt) {
  const char *v = std::getenv(name);
  return v ? (int)std::strtol(v, nullptr, 10) : dflt;
}

const double VoxelSize = envd("KF_REF_VOXEL_SIZE", 0.012);
const double UnknownClipDistance = envd("KF_REF_UNKNOWN_CLIP", VoxelSize * 4);
const double MaxSurfaceVoxelDistance = envd("KF_REF_MAX_SURFACE", VoxelSize * 4);
const bool FUSE_BY_MERGE = true;
const FusionTechnique fusionTechnique = KILLING_FUSION;
const DEFORMABLE_DATASET datasetType = SNOOPY;
const int numImageFiles[2] = {0, 0};
const std::string imageDir[2] = {std::string(""), std::string("")};
const std::string intrinsicParamsFile = "";
const double datasetDepthMinMaxValues[2][2] = {{1.0, 1.0}, {1.0, 1.0}};
const std::string outputDir[2] = {"", ""};
const bool EnergyTypeUsed[3] = {envi("KF_REF_USE_DATA", 1) != 0,
                                envi("KF_REF_USE_LEVELSET", 1) != 0,
                                envi("KF_REF_USE_KILLING", 1) != 0};
const bool UseZeroDisplacementFieldForNextFrame = true;
const bool UpdateAllVoxelsInEachIter = envi("KF_REF_JACOBI", 1) != 0;
const bool UsePreviousIterationDeformationField = true;
const bool UseTrustStrategy = envi("KF_REF_TRUST", 0) != 0;
const double deltaSize = envd("KF_REF_DELTA_SIZE", 0.05);
const int KILLING_MAX_ITERATIONS = envi("KF_REF_ITERATIONS", 1024);
const double threshold = envd("KF_REF_THRESHOLD", 0.000001);
const double alpha = envd("KF_REF_ALPHA", 0.025);
const double omegaKilling = envd("KF_REF_OMEGA_K", 0.04);
const double gammaKilling = envd("KF_REF_GAMMA_K", 0);
const double omegaLevelSet = envd("KF_REF_OMEGA_S", 0.1);
const double epsilon = envd("KF_REF_EPSILON", 0.00001);
