// C++ mirror of gpugi's renderer interface, driving the CUDA library through
// its C ABI (gpugi_cuda.h) instead of OpenGL compute shaders.
//
//   Renderer                 gpugi/renderer/renderer.hpp:25-51
//   RendererSystem           gpugi/renderer/renderersystem.hpp:23-214, renderersystem.cpp:23-260
//   Pathtracer               gpugi/renderer/pathtracer.cpp:20-53
//   LightPathtracer          gpugi/renderer/lightpathtracer.cpp:12-49
//   BidirectionalPathtracer  gpugi/renderer/bidirectionalpathtracer.cpp:20-203
//   Camera                   gpugi/camera/camera.hpp, camera.cpp:76-85
//   Scene                    gpugi/scene/scene.hpp:17-205 (loading from bvhmake's file, not Bim)
//   WritePfm / LoadPfm       gpugi/imageut/hdrimage.cpp:6-66
//   TextureMSE               gpugi/imageut/texturemse.hpp:15-40
//
// Differences a caller sees:
//   * The backbuffer is a DeviceImage (device RGBA32F accumulation, optional
//     FP64 copy) instead of gl::Texture2D; Renderer::SetScreenSize takes it.
//   * The environment is a constant sky colour (Environment) instead of a
//     cubemap texture.
//   * The GlobalConfig "pathLength" parameter is RendererSystem::SetMaxPathLength.
//   * Errors of the CUDA library throw GpugiError (the reference logs and
//     continues on GL errors); a failed call leaves the accumulation as it was
//     before that call's kernels.
//   * One thread makes all calls on one RendererSystem, as with the GL context.
//   * NrcPathtracer (path tracing with the neural radiance cache) has no
//     counterpart in the reference.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpugi_bvhmake.h"
#include "gpugi_cuda.h"

#ifndef GPUGI_HOST_HAVE_EI
// Minimal stand-ins for the epsilon-intersection vector types the reference
// interface uses. Define GPUGI_HOST_HAVE_EI and include <ei/vector.hpp>
// first to use the real ones.
namespace ei {
struct Vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    Vec3() = default;
    Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
struct IVec2 {
    int x = 0, y = 0;
    IVec2() = default;
    IVec2(int a, int b) : x(a), y(b) {}
};
enum class Types3D { BOX, ELLIPSOID, OBOX };
}  // namespace ei
#endif

using uint64 = std::uint64_t;

class GpugiError : public std::runtime_error {
public:
    GpugiError(int status, const std::string& what) : std::runtime_error(what), m_status(status) {}
    int GetStatus() const { return m_status; }

private:
    int m_status;
};

// Headless backbuffer: the accumulation image on the device.
class DeviceImage {
public:
    DeviceImage(gpugi_ctx* ctx, int width, int height, bool fp64 = false);
    ~DeviceImage();
    DeviceImage(const DeviceImage&) = delete;
    DeviceImage& operator=(const DeviceImage&) = delete;

    int GetWidth() const { return m_width; }
    int GetHeight() const { return m_height; }
    bool HasFP64() const { return m_fp64; }
    void ClearToZero();
    // Accumulated sums, row 0 = bottom row of the screen (GL convention).
    std::vector<float> ReadRGBA() const;
    std::vector<double> ReadRGB64() const;
    // Replaces the sums (gpugi_image_write); an empty rgb64 zeroes an FP64 accumulation.
    void Write(const std::vector<float>& rgba, const std::vector<double>& rgb64);
    gpugi_image* GetHandle() const { return m_image; }
    gpugi_ctx* GetContext() const { return m_ctx; }

private:
    gpugi_ctx* m_ctx;
    gpugi_image* m_image = nullptr;
    int m_width, m_height;
    bool m_fp64;
};

// Constant environment radiance (stands in for the cubemap).
struct Environment {
    ei::Vec3 radiance;
};

class Camera {
public:
    Camera();
    Camera(const ei::Vec3& position, const ei::Vec3& lookat, float aspectRatio, float verticalFOV = 60.0f,
           const ei::Vec3& up = ei::Vec3(0.0f, 1.0f, 0.0f));
    virtual ~Camera() = default;

    const ei::Vec3& GetPosition() const { return m_position; }
    const ei::Vec3& GetLookAt() const { return m_lookat; }
    virtual void SetAspectRatio(float aspect) { m_aspectRatio = aspect; }
    virtual void SetVFov(float vfov) { m_yfov = vfov; }
    virtual void SetPosition(const ei::Vec3& position) { m_position = position; }
    virtual void SetLookAt(const ei::Vec3& lookat) { m_lookat = lookat; }
    const ei::Vec3& GetUp() const { return m_up; }
    float GetVFov() const { return m_yfov; }
    float GetAspectRatio() const { return m_aspectRatio; }
    // U and V scaled by tan(vfov/2) * aspect and tan(vfov/2), W unit view direction.
    void ComputeCameraParams(ei::Vec3& cameraU, ei::Vec3& cameraV, ei::Vec3& cameraW) const;

protected:
    ei::Vec3 m_position, m_lookat, m_up;
    float m_yfov;
    float m_aspectRatio;
};

struct PointLight {
    ei::Vec3 position;
    ei::Vec3 intensity;
};

class Scene {
public:
    // Loads bvhmake's NamedArray file: hierarchy, bounding volumes, triangle
    // blocks, vertices {position, normal, texcoord}. Materials come from the
    // scene JSON beside the file (<stem>.json, by the "materialref" names,
    // with Scene::LoadMaterial's mapping), else from the file's
    // "gpugi_materials" chunk, else a single grey Lambertian.
    Scene(gpugi_ctx* ctx, const std::string& file);
    ~Scene();
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    gpugi_scene* GetHandle() const { return m_scene; }
    ei::Types3D GetBvhType() const { return m_bvhType; }
    const char* GetBvhTypeDefineString() const;
    std::uint32_t GetNumTrianglesPerLeaf() const { return m_leafSize; }
    std::uint32_t GetNumLeafTriangles() const { return m_numLeafBlocks * m_leafSize; }
    std::uint32_t GetNumInnerNodes() const { return m_numNodes; }
    std::uint32_t GetNumMaterials() const { return m_numMaterials; }
    std::uint32_t GetNumVertices() const { return m_numVertices; }
    std::uint32_t GetNumTreeLevels() const { return m_maxDepth + 1; }
    // Bounding box of the scene (min, max).
    void GetBoundingBox(ei::Vec3& min, ei::Vec3& max) const {
        min = m_boxMin;
        max = m_boxMax;
    }
    void AddPointLight(const PointLight& light);
    const std::vector<PointLight>& GetPointLights() const { return m_pointLights; }
    // Node NDFs of the file ("approx_sggx", 6 uint16 per node), computed from
    // the vertex normals when the file has none; empty without normals
    // (Scene::GetSGGXBuffer, scene.cpp:127-130).
    const std::vector<std::uint16_t>& GetSGGX() const { return m_sggx; }

private:
    gpugi_ctx* m_ctx;
    gpugi_scene* m_scene = nullptr;
    ei::Types3D m_bvhType = ei::Types3D::BOX;
    std::uint32_t m_leafSize = 0, m_numLeafBlocks = 0, m_numNodes = 0, m_numMaterials = 0, m_numVertices = 0,
                  m_maxDepth = 0;
    ei::Vec3 m_boxMin, m_boxMax;
    std::vector<PointLight> m_pointLights;
    std::vector<std::uint16_t> m_sggx;
};

class RendererSystem;

// Abstract base class of all renderers (gpugi/renderer/renderer.hpp:25-51).
class Renderer {
public:
    virtual ~Renderer() = default;
    virtual std::string GetName() const = 0;
    virtual void SetScene(std::shared_ptr<Scene> scene) {}
    virtual void SetCamera(const Camera& camera) {}
    virtual void SetScreenSize(const DeviceImage& newBackbuffer) = 0;
    virtual void SetEnvironmentMap(std::shared_ptr<Environment> envMap) {}
    // One iteration into the backbuffer; RendererSystem::Draw advances the iteration count.
    virtual void Draw() = 0;
    const RendererSystem& GetRendererSystem() const { return m_rendererSystem; }

protected:
    explicit Renderer(RendererSystem& rendererSystem) : m_rendererSystem(rendererSystem) {}
    RendererSystem& m_rendererSystem;
};

class RendererSystem {
public:
    explicit RendererSystem(int device = 0);
    ~RendererSystem();
    RendererSystem(const RendererSystem&) = delete;
    RendererSystem& operator=(const RendererSystem&) = delete;

    void SetScene(std::shared_ptr<Scene> scene);
    const std::shared_ptr<Scene>& GetScene() const { return m_scene; }
    void SetEnvironmentMap(std::shared_ptr<Environment> env);
    void SetCamera(const Camera& camera);
    const Camera& GetCamera() const { return m_camera; }
    void SetScreenSize(const ei::IVec2& newSize);
    DeviceImage& GetBackbuffer() { return *m_backbuffer; }
    const DeviceImage& GetBackbuffer() const { return *m_backbuffer; }
    Renderer* GetActiveRenderer() { return m_activeRenderer.get(); }

    // Replaces the active renderer: resets the iteration count, clears the
    // backbuffer, then SetScreenSize -> SetCamera -> SetScene -> SetEnvironmentMap.
    template <typename RendererType, typename... Args>
    void SetRenderer(Args&&... arguments) {
        m_activeRenderer.reset();
        ResetIterationCount();
        if (m_backbuffer) m_backbuffer->ClearToZero();
        m_activeRenderer.reset(new RendererType(*this, std::forward<Args>(arguments)...));
        if (m_backbuffer) m_activeRenderer->SetScreenSize(*m_backbuffer);
        m_activeRenderer->SetCamera(m_camera);
        if (m_scene) m_activeRenderer->SetScene(m_scene);
        m_activeRenderer->SetEnvironmentMap(m_envMap);
    }

    // Active renderer's Draw, then PerIterationBufferUpdate; adds the
    // elapsed wall time (after a device synchronisation) to GetRenderTime.
    void Draw();
    unsigned long GetIterationCount() const { return m_iterationCount; }
    uint64 GetRenderTime() const { return m_renderTime; }  // ms
    void SetNumInitialLightSamples(unsigned int numInitialLightSamples);
    unsigned int GetNumInitialLightSamples() const { return m_numInitialLightSamples; }
    void ResetIterationCount();
    // Advances the iteration (optionally) and draws the next set of initial
    // light samples from the light sampler.
    void PerIterationBufferUpdate(bool iterationIncrement = true);

    // Checkpoint of a long accumulation (an addition: the reference only
    // saves the normalised backbuffer, Application::SaveImage,
    // application.cpp:394-414). Writes <base>.pfm (the average, as SaveImage
    // does), <base>.accum (the exact sums: height x width RGBA float32, then
    // height x width RGB float64 with an FP64 backbuffer, little-endian) and
    // <base>.json (size, iteration count, the frame index of the next
    // iteration, the light sampler's state for the next iteration's light
    // samples, the active renderer and the settings).
    bool SaveCheckpoint(const std::string& base) const;
    // Restores the sums, the iteration count and the light sampler from a
    // checkpoint of the same screen size and renderer, so that further Draw
    // calls continue the same estimator. Throws GpugiError on a mismatch.
    void LoadCheckpoint(const std::string& base);

    // Parameters the reference keeps in GlobalConfig and shader defines.
    void SetMaxPathLength(unsigned int pathLength) { m_maxPathLength = pathLength; }
    unsigned int GetMaxPathLength() const { return m_maxPathLength; }
    void SetRussianRouletteStart(unsigned int depth) { m_rrStartDepth = depth; }
    unsigned int GetRussianRouletteStart() const { return m_rrStartDepth; }
    // Random streams of the passes: per-pixel PCG (default) or, with true,
    // gpugi's own wanghash + xorshift32 streams (GPUGI_RENDER_REFERENCE_RNG).
    void SetReferenceRandomStreams(bool reference) { m_referenceRng = reference; }
    bool GetReferenceRandomStreams() const { return m_referenceRng; }

    // Access for the renderers.
    gpugi_ctx* GetContext() const { return m_ctx; }
    const gpugi_camera& GetCameraParams() const { return m_cameraParams; }
    const float* GetInitialLightSamples() const { return m_lightSamples.data(); }
    ei::Vec3 GetSkyRadiance() const { return m_envMap ? m_envMap->radiance : ei::Vec3(); }
    // Parameters of one iteration of a pass at the current state.
    gpugi_render_params MakeRenderParams(gpugi_pass pass) const;
    void Check(gpugi_status status) const;

private:
    void UpdateCameraParams();

    gpugi_ctx* m_ctx = nullptr;
    std::unique_ptr<DeviceImage> m_backbuffer;
    Camera m_camera;
    gpugi_camera m_cameraParams{};
    unsigned long m_iterationCount = 0;
    uint64 m_renderTime = 0;
    std::shared_ptr<Scene> m_scene;
    std::shared_ptr<Environment> m_envMap;
    unsigned int m_numInitialLightSamples = 0;
    std::vector<float> m_lightSamples;  // 8 floats per initial light sample
    uint64_t m_lightSamplerState = 123;  // LightSampler's xorshift state
    uint64_t m_lightSamplerStateBefore = 123;  // the state that drew m_lightSamples
    unsigned int m_maxPathLength = 8;
    unsigned int m_rrStartDepth = 0;
    bool m_referenceRng = false;
    std::unique_ptr<Renderer> m_activeRenderer;
};

class Pathtracer : public Renderer {
public:
    explicit Pathtracer(RendererSystem& rendererSystem);
    std::string GetName() const override { return "Pathtracer"; }
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
};

class LightPathtracer : public Renderer {
public:
    explicit LightPathtracer(RendererSystem& rendererSystem);
    std::string GetName() const override { return "LightPathtracer"; }
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
};

class BidirectionalPathtracer : public Renderer {
public:
    explicit BidirectionalPathtracer(RendererSystem& rendererSystem);
    std::string GetName() const override { return "BidirectionalPathtracer"; }
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
};

// PhotonMapper (gpugi/renderer/photonmapper.hpp): a photon map per iteration,
// gathered at the first diffuse decision of the eye paths. The settings are
// the GlobalConfig parameters pm_nphotons, pm_r and pm_progressive.
class PhotonMapper : public Renderer {
public:
    explicit PhotonMapper(RendererSystem& rendererSystem);
    std::string GetName() const override { return "PhotonMapper"; }
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
    void SetNumPhotonsPerLightSample(unsigned int n) { m_numPhotonsPerLightSample = n; }
    void SetQueryRadius(float r) { m_queryRadius = r; }
    void SetProgressiveRadius(bool on) { m_progressiveRadius = on; }

private:
    unsigned int m_numPhotonsPerLightSample = 1u << 11;
    float m_queryRadius = 0.01f;
    bool m_progressiveRadius = false;
};

// PixelMapLighttracer (gpugi/renderer/pixelmaplighttracer.hpp): an importon
// map per iteration from the eye paths' diffuse decisions behind specular
// bounces, photons splatting into it and reprojecting against a G-buffer.
// The settings are the GlobalConfig parameters im_nphotons, im_r and
// im_progressive.
class PixelMapLighttracer : public Renderer {
public:
    explicit PixelMapLighttracer(RendererSystem& rendererSystem);
    std::string GetName() const override { return "PixelMapLighttracer"; }
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
    void SetNumPhotonsPerLightSample(unsigned int n) { m_numPhotonsPerLightSample = n; }
    void SetQueryRadius(float r) { m_queryRadius = r; }
    void SetProgressiveRadius(bool on) { m_progressiveRadius = on; }

private:
    unsigned int m_numPhotonsPerLightSample = 1u << 11;
    float m_queryRadius = 0.005f;
    bool m_progressiveRadius = false;
};

// WhittedRayTracer (gpugi/renderer/whittedraytracer.hpp): follows specular and
// glossy decisions, ends at the first diffuse decision with two NEE samples.
class WhittedRayTracer : public Renderer {
public:
    explicit WhittedRayTracer(RendererSystem& rendererSystem);
    std::string GetName() const override { return "WhittedRayTracer"; }
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
};

// HierarchyImportance (gpugi/renderer/hierarchyimportance.hpp): at the first
// iteration after a camera change, the importance of every hierarchy node
// for this view; then a path tracer of at most 4 vertices whose walks stop
// at nodes that stand in well for their subtree, shading them with the
// node's averaged material and a normal from its NDF. Needs node NDFs and
// an AABB hierarchy.
class HierarchyImportance : public Renderer {
public:
    explicit HierarchyImportance(RendererSystem& rendererSystem);
    std::string GetName() const override { return "HierarchyImportance"; }
    void SetScene(std::shared_ptr<Scene> scene) override;
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
};

// Path tracer whose camera paths end in the neural radiance cache, trained
// online on a fraction of full-length paths of every iteration.
struct NrcSettings {
    unsigned int terminateDepth = 1;
    float trainFraction = 0.03f;
    unsigned int maxTrainSamples = 65536;
    unsigned int trainSteps = 1;
    float learningRate = 1e-2f;
    uint64_t seed = 1;
};

class NrcPathtracer : public Renderer {
public:
    explicit NrcPathtracer(RendererSystem& rendererSystem, const NrcSettings& settings = NrcSettings());
    ~NrcPathtracer() override;
    std::string GetName() const override { return "NrcPathtracer"; }
    void SetScene(std::shared_ptr<Scene> scene) override;
    void SetScreenSize(const DeviceImage&) override {}
    void Draw() override;
    // Continue training while drawing (default) or use the cache as it is.
    void SetTraining(bool train) { m_train = train; }
    gpugi_nrc* GetCache() const { return m_nrc; }

protected:
    NrcPathtracer(RendererSystem& rendererSystem, const NrcSettings& settings, gpugi_pass pass);

private:
    NrcSettings m_settings;
    gpugi_nrc* m_nrc = nullptr;
    bool m_train = true;
    gpugi_pass m_pass = GPUGI_PASS_PT;
};

// Bidirectional path tracer whose eye paths end in the radiance cache at
// vertex terminateDepth; shorter paths keep BPT's strategies, extra PT
// training paths (trainFraction of the pixels) feed the cache.
class NrcBidirectionalPathtracer : public NrcPathtracer {
public:
    explicit NrcBidirectionalPathtracer(RendererSystem& rendererSystem, const NrcSettings& settings = NrcSettings())
        : NrcPathtracer(rendererSystem, settings, GPUGI_PASS_BPT) {}
    std::string GetName() const override { return "NrcBidirectionalPathtracer"; }
};

// imageut: RGB PFM files; rows bottom-up as the backbuffer stores them.
bool WritePfm(const float* rgba, const ei::IVec2& size, const std::string& filename, std::uint32_t divisor);
std::unique_ptr<float[]> LoadPfm(const std::string& filename, ei::IVec2& size);  // 3 floats per pixel

// Mean over pixels of |rgb / divisor - reference|^2, reduced in FP64 on the device.
class TextureMSE {
public:
    bool HasValidReferenceImage() const { return !m_reference.empty(); }
    void LoadReferenceFromPFM(const std::string& filename);
    float ComputeCurrentMSE(const DeviceImage& texture, unsigned int divisor);
    double ComputeCurrentMSE64(const DeviceImage& texture, unsigned int divisor);

private:
    std::vector<float> m_reference;
    ei::IVec2 m_size;
};
