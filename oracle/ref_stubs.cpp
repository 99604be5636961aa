// The reference's CUDA driver entry points (resources/cuda/**), which the
// checker build of its CPU code links against but never calls: each aborts.
// TEST INFRASTRUCTURE ONLY.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <GLM/glm.hpp>

#include "DataStructures/GpuMesh.h"
#include "DataStructures/Mesh.h"
#include "DataStructures/NodeGroups.h"

[[noreturn]] static void cuda_driver_called(const char* f)
{
    std::fprintf(stderr, "checker build: the reference CUDA driver %s is not available\n", f);
    std::abort();
}

bool verboseCuda = true;
void installCudaMeanRatioEvaluator() { cuda_driver_called("installCudaMeanRatioEvaluator"); }
void installCudaMetricConformityEvaluator() { cuda_driver_called("installCudaMetricConformityEvaluator"); }
void installCudaMetricFreeMeasurer() { cuda_driver_called("installCudaMetricFreeMeasurer"); }
void installCudaMetricWiseMeasurer() { cuda_driver_called("installCudaMetricWiseMeasurer"); }
void installCudaAnalyticSampler() { cuda_driver_called("installCudaAnalyticSampler"); }
void installCudaUniformSampler() { cuda_driver_called("installCudaUniformSampler"); }
void installCudaLocalSampler() { cuda_driver_called("installCudaLocalSampler"); }
void updateCudaLocalTets(const std::vector<GpuLocalTet>&) { cuda_driver_called("updateCudaLocalTets"); }
void updateCudaLocalCache(const std::vector<GLuint>&) { cuda_driver_called("updateCudaLocalCache"); }
void updateCudaRefVerts(const std::vector<GpuVert>&) { cuda_driver_called("updateCudaRefVerts"); }
void updateCudaRefMetrics(const std::vector<GpuMetric>&) { cuda_driver_called("updateCudaRefMetrics"); }
void installCudaKdTreeSampler() { cuda_driver_called("installCudaKdTreeSampler"); }
void updateCudaKdNodes(const std::vector<GpuKdNode>&) { cuda_driver_called("updateCudaKdNodes"); }
void installCudaTextureSampler() { cuda_driver_called("installCudaTextureSampler"); }
void updateCudaSamplerTextures(const std::vector<glm::vec4>&, const std::vector<glm::vec4>&, const glm::mat4&,
                               const glm::ivec3)
{
    cuda_driver_called("updateCudaSamplerTextures");
}
void installCudaGetmeSmoother() { cuda_driver_called("installCudaGetmeSmoother"); }
void installCudaNelderMeadSmoother(float, int, float, float, float, float, float)
{
    cuda_driver_called("installCudaNelderMeadSmoother");
}
void installCudaGradientDescentSmoother(int, float) { cuda_driver_called("installCudaGradientDescentSmoother"); }
void installCudaSpringLaplaceSmoother(float) { cuda_driver_called("installCudaSpringLaplaceSmoother"); }
void installCudaQualityLaplaceSmoother(float) { cuda_driver_called("installCudaQualityLaplaceSmoother"); }
void installCudaSpawnSearchSmoother(float, const std::vector<glm::vec4>)
{
    cuda_driver_called("installCudaSpawnSearchSmoother");
}
void setCudaMetricScaling(double) { cuda_driver_called("setCudaMetricScaling"); }
void setCudaMetricScalingSqr(double) { cuda_driver_called("setCudaMetricScalingSqr"); }
void setCudaMetricScalingCube(double) { cuda_driver_called("setCudaMetricScalingCube"); }
void setCudaMetricAspectRatio(double) { cuda_driver_called("setCudaMetricAspectRatio"); }
void setCudaRotMat(const glm::dmat3&, const glm::dmat3&) { cuda_driver_called("setCudaRotMat"); }
void smoothCudaVertices(const NodeGroups::GpuDispatch&) { cuda_driver_called("smoothCudaVertices"); }
void smoothCudaSpawnVertices(const NodeGroups::GpuDispatch&) { cuda_driver_called("smoothCudaSpawnVertices"); }
void fetchCudaSubsurfaceVertices(std::vector<MeshVert>&, const NodeGroups::ParallelGroup&)
{
    cuda_driver_called("fetchCudaSubsurfaceVertices");
}
void sendCudaBoundaryVertices(const std::vector<MeshVert>&, const NodeGroups::ParallelGroup&)
{
    cuda_driver_called("sendCudaBoundaryVertices");
}

class QualityHistogram;
void evaluateCudaMeshQuality(size_t, size_t, QualityHistogram&) { cuda_driver_called("evaluateCudaMeshQuality"); }
