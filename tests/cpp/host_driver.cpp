// Test driver for the C++ class layer (SDF, DisplacementField,
// KillingFusion, DatasetReader, SimpleMesh).  The Python tests compile it,
// run one mode and compare the files it writes with the oracle.
//
//   host_driver spheres <outdir> <solver> <iterations>
//       KillingFusion::processTest(1), (2) and (3) on the two-sphere sample
//       (needs a dataset only for the constructor: <outdir>/dataset)
//   host_driver dataset <root> <outdir> <solver> <iterations> <frames> <voxel>
//       processNextFrame over <frames> frames; writes the three meshes of each
//       frame (OFF), psi of each frame and the final canonical SDF (.bin)
//   host_driver process <root> <outdir> <solver> <iterations> <voxel>
//       KillingFusion::process: psi carried over, fusion through psi
//   host_driver refdataset <root> <outdir> <solver> <iterations> <frames>
//       the same on the reference's PNG dataset layout and default config
//   host_driver points <outdir>
//       point queries of SDF and DisplacementField on a small seeded grid
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "KillingFusion.h"

static kf_solver solver_of(const char *s) {
  if (!std::strcmp(s, "exact")) return KF_SOLVER_EXACT;
  if (!std::strcmp(s, "plain")) return KF_SOLVER_PLAIN;
  if (!std::strcmp(s, "band")) return KF_SOLVER_BAND;
  return KF_SOLVER_FUSED;
}

static void write_mesh(SimpleMesh *m, const std::string &path) {
  if (!m) return;
  if (!m->WriteMesh(path)) throw std::runtime_error("cannot write " + path);
  delete m;
}

static int run_spheres(int argc, char **argv) {
  if (argc < 5) return 2;
  std::string out = std::string(argv[2]) + "/";
  kf::config().solver = solver_of(argv[3]);
  kf::config().KILLING_MAX_ITERATIONS = std::atoi(argv[4]);
  if (argc > 5 && !std::strcmp(argv[5], "trust")) {
    // the data term alone with the trust-region step (config.cpp:23, 27)
    kf::Config &c = kf::config();
    c.EnergyTypeUsed[1] = c.EnergyTypeUsed[2] = false;
    c.UseTrustStrategy = true;
    c.alpha = std::atof(argv[6]);
  }
  SDF::outputDir() = out;
  KillingFusion fusion{DatasetReader(out + "dataset")};
  fusion.processTest(1);
  fusion.processTest(2);
  fusion.processTest(3);
  std::cout << "solve iterations " << fusion.lastSolveStats().iterations_run << std::endl;
  return 0;
}

static int run_dataset(int argc, char **argv) {
  if (argc < 8) return 2;
  std::string root = argv[2], out = std::string(argv[3]) + "/";
  kf::Config &c = kf::config();
  c.solver = solver_of(argv[4]);
  c.KILLING_MAX_ITERATIONS = std::atoi(argv[5]);
  const int frames = std::atoi(argv[6]);
  c.VoxelSize = std::atof(argv[7]);
  c.UnknownClipDistance = c.VoxelSize * 5;
  c.MaxSurfaceVoxelDistance = c.VoxelSize * 5;
  // paper weights (config.cpp:32-41 comment)
  c.alpha = 0.1;
  c.omegaKilling = 0.5;
  c.gammaKilling = 0.1;
  c.omegaLevelSet = 0.2;
  SDF::outputDir() = out;
  KillingFusion fusion{DatasetReader(root)};
  fusion.setFrameRange(0, frames);
  const char *names[3] = {"live", "registered", "canonical"};
  for (int f = 0; f < frames; ++f) {
    std::vector<SimpleMesh *> meshes = fusion.processNextFrame();
    for (int k = 0; k < 3; ++k) {
      char name[256];
      std::snprintf(name, sizeof name, "%s%s_%03d.off", out.c_str(), names[k], f);
      write_mesh(meshes[k], name);
    }
    char name[256];
    std::snprintf(name, sizeof name, "%spsi_%03d.bin", out.c_str(), f);
    fusion.getCurrentFrameDisplacementField()->dumpToBinFile(name);
  }
  fusion.getCanonicalSdf()->dumpToBinFile(out + "canonical.bin", c.UnknownClipDistance, 1.0);
  std::cout << "frame index " << fusion.getCurrentFrameIndex() << std::endl;
  return 0;
}

// KillingFusion::process over a raw dataset (frames 4 .. numFrames-1, psi
// carried from frame to frame, fused through psi):
//   host_driver process <root> <outdir> <solver> <iterations> <voxel>
static int run_process(int argc, char **argv) {
  if (argc < 7) return 2;
  std::string root = argv[2], out = std::string(argv[3]) + "/";
  kf::Config &c = kf::config();
  c.solver = solver_of(argv[4]);
  c.KILLING_MAX_ITERATIONS = std::atoi(argv[5]);
  c.VoxelSize = std::atof(argv[6]);
  c.UnknownClipDistance = c.MaxSurfaceVoxelDistance = c.VoxelSize * 5;
  SDF::outputDir() = out;
  KillingFusion fusion{DatasetReader(root)};
  fusion.process();
  return 0;
}

// The reference's own dataset layout (Snoopy/, PNG depth and mask,
// intrinsics_kinect1.txt) with the reference's default configuration:
//   host_driver process <root> <outdir> <solver> <iterations> <voxel>
//       KillingFusion::process: psi carried over, fusion through psi
//   host_driver refdataset <root> <outdir> <solver> <iterations> <frames>
static int run_refdataset(int argc, char **argv) {
  if (argc < 7) return 2;
  std::string root = argv[2], out = std::string(argv[3]) + "/";
  kf::Config &c = kf::config();
  c.solver = solver_of(argv[4]);
  c.KILLING_MAX_ITERATIONS = std::atoi(argv[5]);
  const int frames = std::atoi(argv[6]);
  c.datasetType = 1;
  SDF::outputDir() = out;
  DatasetReader reader(root);
  if (!reader.referenceLayout()) throw std::runtime_error("expected the reference's layout");
  std::cout << "frames " << reader.getNumImageFiles() << " depth " << reader.getMinimumDepthThreshold() << " "
            << reader.getMaximumDepthThreshold() << std::endl;
  KillingFusion fusion{reader};
  fusion.setFrameRange(0, frames);
  const char *names[3] = {"live", "registered", "canonical"};
  for (int f = 0; f < frames; ++f) {
    std::vector<SimpleMesh *> meshes = fusion.processNextFrame();
    for (int k = 0; k < 3; ++k) {
      char name[256];
      std::snprintf(name, sizeof name, "%s%s_%03d.off", out.c_str(), names[k], f);
      write_mesh(meshes[k], name);
    }
    char name[256];
    std::snprintf(name, sizeof name, "%spsi_%03d.bin", out.c_str(), f);
    fusion.getCurrentFrameDisplacementField()->dumpToBinFile(name);
  }
  fusion.getCanonicalSdf()->dumpToBinFile(out + "canonical.bin", c.UnknownClipDistance, 1.0);
  return 0;
}

// Point queries on a grid and psi read from <outdir>/grid.f32 (nx ny nz,
// then phi) and <outdir>/psi.bin (the DisplacementField format), at the
// points in <outdir>/points.f64 (n, then n xyz triples) and the voxels in
// <outdir>/voxels.i32 (n, then n xyz triples).  Writes <outdir>/queries.f64.
static int run_points(int argc, char **argv) {
  if (argc < 3) return 2;
  std::string out = std::string(argv[2]) + "/";
  kf::Config &c = kf::config();
  c.VoxelSize = 0.004;
  c.UnknownClipDistance = c.MaxSurfaceVoxelDistance = 0.02;
  std::ifstream g(out + "grid.f32", std::ios::binary);
  if (!g) throw std::runtime_error("cannot open " + out + "grid.f32");
  int dims[3];
  g.read((char *)dims, sizeof dims);
  const size_t N = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<float> phi(N);
  std::vector<int32_t> w(N);
  g.read((char *)phi.data(), N * sizeof(float));
  g.read((char *)w.data(), N * sizeof(int32_t));
  kf::Vec3d mn(0, 0, 0);
  kf::Vec3d mx((dims[0] - 0.5) * c.VoxelSize, (dims[1] - 0.5) * c.VoxelSize, (dims[2] - 0.5) * c.VoxelSize);
  SDF sdf(c.VoxelSize, mn, mx, c.UnknownClipDistance);
  kf::check(kf_grid_upload(sdf.handle(), phi.data(), w.data(), nullptr), "upload");
  DisplacementField psi = DisplacementField::loadFromBinFile(out + "psi.bin");
  std::ifstream pf(out + "points.f64", std::ios::binary);
  std::ifstream vf(out + "voxels.i32", std::ios::binary);
  if (!pf || !vf) throw std::runtime_error("cannot open the query files in " + out);
  int np = 0;
  pf.read((char *)&np, sizeof np);
  std::vector<double> pts(3 * (size_t)np);
  pf.read((char *)pts.data(), pts.size() * sizeof(double));
  int nv = 0;
  vf.read((char *)&nv, sizeof nv);
  std::vector<int32_t> vox(3 * (size_t)nv);
  vf.read((char *)vox.data(), vox.size() * sizeof(int32_t));
  std::vector<double> res;
  for (int i = 0; i < np; ++i) {
    kf::Vec3d p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    res.push_back(sdf.getDistance(p));
    res.push_back(sdf.getWeight(p));
    kf::Vec3d g3 = sdf.computeDistanceGradient(p);
    for (int k = 0; k < 3; ++k) res.push_back(g3(k));
    kf::Mat3d H = sdf.computeDistanceHessian(p);
    for (int k = 0; k < 9; ++k) res.push_back(H.m[k]);
    kf::Vec3d d = psi.getDisplacementAtf(p);
    for (int k = 0; k < 3; ++k) res.push_back(d(k));
    res.push_back(sdf.getDistancef(p, &psi));
    kf::Mat3d J = psi.computeJacobian(p(0), p(1), p(2));
    for (int k = 0; k < 9; ++k) res.push_back(J.m[k]);
    res.push_back(psi.computeKillingEnergy(p(0), p(1), p(2)));
  }
  for (int i = 0; i < nv; ++i) {
    kf::Vec3i v(vox[3 * i], vox[3 * i + 1], vox[3 * i + 2]);
    res.push_back(sdf.getDistanceAtIndex(v));
    res.push_back((double)sdf.getWeightAtIndex(v));
    res.push_back(sdf.getDistance(v, &psi));
    res.push_back(sdf.getWeight(v, &psi));
    kf::Vec3d g3 = sdf.computeDistanceGradient(v, &psi);
    for (int k = 0; k < 3; ++k) res.push_back(g3(k));
    kf::Mat3d H = sdf.computeDistanceHessian(v, &psi);
    for (int k = 0; k < 9; ++k) res.push_back(H.m[k]);
    kf::Vec3d d = psi.getDisplacementAt(v);
    for (int k = 0; k < 3; ++k) res.push_back(d(k));
    kf::Vec3d kg = psi.computeKillingEnergyGradient2(v);
    for (int k = 0; k < 3; ++k) res.push_back(kg(k));
  }
  std::ofstream o(out + "queries.f64", std::ios::binary);
  o.write((const char *)res.data(), res.size() * sizeof(double));
  return 0;
}

// The reference's public self-tests, run on the drop-in classes.
static int run_selftests() {
  SDF::testGetDistance();
  SDF::testGetWeight();
  SDF::testComputeDistanceGradient();
  SDF::testComputeDistanceHessian();
  DisplacementField::testJacobian();
  DisplacementField::testKillingEnergy();
  std::cout << "selftests ok" << std::endl;
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  try {
    if (!std::strcmp(argv[1], "spheres")) return run_spheres(argc, argv);
    if (!std::strcmp(argv[1], "dataset")) return run_dataset(argc, argv);
    if (!std::strcmp(argv[1], "refdataset")) return run_refdataset(argc, argv);
    if (!std::strcmp(argv[1], "process")) return run_process(argc, argv);
    if (!std::strcmp(argv[1], "points")) return run_points(argc, argv);
    if (!std::strcmp(argv[1], "selftests")) return run_selftests();
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << std::endl;
    return 1;
  } catch (int code) {
    std::cerr << "error code " << code << std::endl;
    return 1;
  }
  return 2;
}
