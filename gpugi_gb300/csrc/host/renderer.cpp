// Implementation of the C++ renderer interface (gpugi_renderer.hpp) over the
// C ABI of the CUDA library.
#include "gpugi_renderer.hpp"

#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>

namespace {

void check_status(gpugi_ctx* ctx, gpugi_status st, const char* what) {
    if (st != GPUGI_OK) {
        const char* msg = ctx ? gpugi_last_error(ctx) : "";
        throw GpugiError((int)st, std::string(what) + ": " + (msg ? msg : ""));
    }
}

ei::Vec3 sub(const ei::Vec3& a, const ei::Vec3& b) { return ei::Vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
ei::Vec3 scale(const ei::Vec3& a, float s) { return ei::Vec3(a.x * s, a.y * s, a.z * s); }
ei::Vec3 cross(const ei::Vec3& a, const ei::Vec3& b) {
    return ei::Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
float len(const ei::Vec3& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
ei::Vec3 normalize(const ei::Vec3& a) { return scale(a, 1.0f / len(a)); }

}  // namespace

// ---------------------------------------------------------------- DeviceImage
DeviceImage::DeviceImage(gpugi_ctx* ctx, int width, int height, bool fp64)
    : m_ctx(ctx), m_width(width), m_height(height), m_fp64(fp64) {
    if (width <= 0 || height <= 0) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "image size must be positive");
    check_status(ctx, gpugi_image_create(ctx, (uint32_t)width, (uint32_t)height, fp64 ? 1u : 0u, &m_image),
                 "gpugi_image_create");
}

DeviceImage::~DeviceImage() { gpugi_image_destroy(m_image); }

void DeviceImage::ClearToZero() { check_status(m_ctx, gpugi_image_clear(m_ctx, m_image), "gpugi_image_clear"); }

std::vector<float> DeviceImage::ReadRGBA() const {
    std::vector<float> out((size_t)m_width * m_height * 4);
    check_status(m_ctx, gpugi_image_read(m_ctx, m_image, out.data(), nullptr), "gpugi_image_read");
    return out;
}

std::vector<double> DeviceImage::ReadRGB64() const {
    if (!m_fp64) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "image has no FP64 accumulation");
    std::vector<double> out((size_t)m_width * m_height * 3);
    check_status(m_ctx, gpugi_image_read(m_ctx, m_image, nullptr, out.data()), "gpugi_image_read");
    return out;
}

void DeviceImage::Write(const std::vector<float>& rgba, const std::vector<double>& rgb64) {
    const size_t n = (size_t)m_width * m_height;
    if (rgba.size() != 4 * n || !(rgb64.empty() || rgb64.size() == 3 * n))
        throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "image data of the wrong size");
    check_status(m_ctx, gpugi_image_write(m_ctx, m_image, rgba.data(), rgb64.empty() ? nullptr : rgb64.data()),
                 "gpugi_image_write");
}

// --------------------------------------------------------------------- Camera
Camera::Camera() : m_position(), m_lookat(), m_up(), m_yfov(0.0f), m_aspectRatio(1.0f) {}

Camera::Camera(const ei::Vec3& position, const ei::Vec3& lookat, float aspectRatio, float verticalFOV,
               const ei::Vec3& up)
    : m_position(position), m_lookat(lookat), m_up(up), m_yfov(verticalFOV), m_aspectRatio(aspectRatio) {}

// camera.cpp:76-85
void Camera::ComputeCameraParams(ei::Vec3& cameraU, ei::Vec3& cameraV, ei::Vec3& cameraW) const {
    cameraW = normalize(sub(m_lookat, m_position));
    cameraU = normalize(cross(cameraW, m_up));
    cameraV = normalize(cross(cameraU, cameraW));
    const float f = std::tan(m_yfov / 2.0f * (3.14159265358979f / 180.0f));
    cameraU = scale(cameraU, f * m_aspectRatio);
    cameraV = scale(cameraV, f);
}

// ---------------------------------------------------------------------- Scene
Scene::Scene(gpugi_ctx* ctx, const std::string& file) : m_ctx(ctx) {
    gpugi_bvh* bvh = nullptr;
    if (gpugi_bvh_read_file(file.c_str(), &bvh) != 0)
        throw GpugiError(GPUGI_ERROR_INVALID_SCENE, std::string("cannot load ") + file + ": " + gpugi_bvh_last_error());
    std::unique_ptr<gpugi_bvh, void (*)(gpugi_bvh*)> guard(bvh, gpugi_bvh_free);
    uint32_t boundsKind = 0;
    gpugi_bvh_info(bvh, &m_numNodes, &m_numLeafBlocks, &m_leafSize, &boundsKind, &m_maxDepth);
    m_bvhType = boundsKind == GPUGI_FIT_ELLIPSOID ? ei::Types3D::ELLIPSOID
                : boundsKind == GPUGI_FIT_OBOX    ? ei::Types3D::OBOX
                                                  : ei::Types3D::BOX;
    std::vector<float> hierarchy((size_t)m_numNodes * (boundsKind == GPUGI_FIT_OBOX ? 12 : 8));
    std::vector<int32_t> slots((size_t)m_numLeafBlocks * m_leafSize * 4);
    gpugi_bvh_export(bvh, hierarchy.data(), slots.data(), nullptr);
    gpugi_bvh_vertices(bvh, &m_numVertices, nullptr);
    std::vector<float> positions((size_t)m_numVertices * 3), normals((size_t)m_numVertices * 3),
        texcoords((size_t)m_numVertices * 2);
    gpugi_bvh_vertices(bvh, &m_numVertices, positions.data());
    gpugi_bvh_vertex_attributes(bvh, normals.data(), texcoords.data());
    // VertexInfo {atan2(n.y, n.x), n.z, u, v} (scene.cpp:79-84)
    std::vector<float> vinfo((size_t)m_numVertices * 4);
    for (size_t v = 0; v < m_numVertices; ++v) {
        vinfo[4 * v] = std::atan2(normals[3 * v + 1], normals[3 * v]);
        vinfo[4 * v + 1] = normals[3 * v + 2];
        vinfo[4 * v + 2] = texcoords[2 * v];
        vinfo[4 * v + 3] = texcoords[2 * v + 1];
    }
    // Materials: the scene JSON next to the file (<stem>.json, as bvhmake
    // writes it) looked up by the "materialref" names, as Scene::LoadMaterial
    // does; else the file's "gpugi_materials" chunk; else one grey Lambertian.
    std::vector<float> materials;
    const uint32_t numNames = gpugi_bvh_num_material_names(bvh);
    const size_t dot = file.find_last_of('.');
    const std::string jsonPath = (dot == std::string::npos ? file : file.substr(0, dot)) + ".json";
    std::ifstream json(jsonPath, std::ios::binary);
    if (numNames && json) {
        const std::string text((std::istreambuf_iterator<char>(json)), std::istreambuf_iterator<char>());
        std::vector<const char*> names(numNames);
        for (uint32_t i = 0; i < numNames; ++i) names[i] = gpugi_bvh_material_name(bvh, i);
        materials.resize((size_t)numNames * 24);
        if (gpugi_materials_from_json(text.c_str(), names.data(), numNames, materials.data()) != 0)
            throw GpugiError(GPUGI_ERROR_INVALID_SCENE, jsonPath + ": " + gpugi_materials_json_error());
        m_numMaterials = numNames;
    } else {
        gpugi_bvh_materials(bvh, &m_numMaterials, nullptr);
        materials.resize((size_t)m_numMaterials * 24);
        if (m_numMaterials) gpugi_bvh_materials(bvh, &m_numMaterials, materials.data());
    }
    if (!m_numMaterials) {
        // one grey Lambertian: diffuse 0.5, ior 1.5, opacity 1, reflectiveness 1 (exponent 1), fresnel (0, 1)
        m_numMaterials = 1;
        materials.assign(24, 0.0f);
        materials[0] = materials[1] = materials[2] = 0.5f;
        materials[3] = 1.5f;
        materials[4] = materials[5] = materials[6] = 1.0f;
        materials[8] = materials[9] = materials[10] = 1.0f;
        materials[11] = 1.0f;
        materials[20] = materials[21] = materials[22] = 1.0f;
    }
    // scene box = root node bounds (AABB: min/max; ellipsoid: center +- radii)
    if (m_numNodes) {
        const float* r = hierarchy.data();
        if (m_bvhType == ei::Types3D::BOX) {
            m_boxMin = ei::Vec3(r[0], r[1], r[2]);
            m_boxMax = ei::Vec3(r[4], r[5], r[6]);
        } else if (m_bvhType == ei::Types3D::OBOX) {  // a cube around the oriented root box
            const float e = std::sqrt(r[4] * r[4] + r[5] * r[5] + r[6] * r[6]);
            m_boxMin = ei::Vec3(r[0] - e, r[1] - e, r[2] - e);
            m_boxMax = ei::Vec3(r[0] + e, r[1] + e, r[2] + e);
        } else {
            m_boxMin = ei::Vec3(r[0] - r[4], r[1] - r[5], r[2] - r[6]);
            m_boxMax = ei::Vec3(r[0] + r[4], r[1] + r[5], r[2] + r[6]);
        }
    }
    bool haveNormals = false;
    for (float n : normals) haveNormals |= n != 0.0f;
    if (haveNormals) {
        m_sggx.resize((size_t)m_numNodes * 6);
        if (gpugi_bvh_sggx(bvh, m_sggx.data()) != 0) m_sggx.clear();
    }
    check_status(ctx,
                 gpugi_scene_upload(ctx, hierarchy.data(), m_numNodes, boundsKind, slots.data(),
                                    (uint32_t)(slots.size() / 4), m_leafSize, positions.data(), vinfo.data(),
                                    m_numVertices, reinterpret_cast<const gpugi_material*>(materials.data()),
                                    m_numMaterials, &m_scene),
                 "gpugi_scene_upload");
}

Scene::~Scene() { gpugi_scene_destroy(m_scene); }

const char* Scene::GetBvhTypeDefineString() const {
    // Scene::GetBvhTypeDefineString (scene.cpp:66-72): AABOX_BVH / OBOX_BVH
    return m_bvhType == ei::Types3D::ELLIPSOID ? "#define BOUNDINGBOX_ELLIPSOID\n"
           : m_bvhType == ei::Types3D::OBOX    ? "#define OBOX_BVH\n"
                                               : "#define BOUNDINGBOX_BOX\n";
}

void Scene::AddPointLight(const PointLight& light) {
    const float p[3] = {light.position.x, light.position.y, light.position.z};
    const float i[3] = {light.intensity.x, light.intensity.y, light.intensity.z};
    check_status(m_ctx, gpugi_scene_add_point_light(m_scene, p, i), "gpugi_scene_add_point_light");
    m_pointLights.push_back(light);
}

// ------------------------------------------------------------- RendererSystem
RendererSystem::RendererSystem(int device) {
    gpugi_opts opts{device, 0};
    check_status(nullptr, gpugi_create(&m_ctx, &opts), "gpugi_create");
}

RendererSystem::~RendererSystem() {
    m_activeRenderer.reset();
    m_backbuffer.reset();
    m_scene.reset();
    gpugi_destroy(m_ctx);
}

void RendererSystem::Check(gpugi_status status) const { check_status(m_ctx, status, "gpugi"); }

void RendererSystem::SetScene(std::shared_ptr<Scene> scene) {
    m_scene = std::move(scene);
    PerIterationBufferUpdate(false);
    m_iterationCount = 0;
    m_renderTime = 0;
    if (m_backbuffer) m_backbuffer->ClearToZero();
    if (m_activeRenderer) m_activeRenderer->SetScene(m_scene);
}

void RendererSystem::SetEnvironmentMap(std::shared_ptr<Environment> env) {
    m_envMap = std::move(env);
    if (m_activeRenderer) m_activeRenderer->SetEnvironmentMap(m_envMap);
}

void RendererSystem::UpdateCameraParams() {
    ei::Vec3 U, V, W;
    m_camera.ComputeCameraParams(U, V, W);
    const ei::Vec3& p = m_camera.GetPosition();
    const float v[12] = {U.x, U.y, U.z, V.x, V.y, V.z, W.x, W.y, W.z, p.x, p.y, p.z};
    std::memcpy(m_cameraParams.U, v, sizeof m_cameraParams.U);
    std::memcpy(m_cameraParams.V, v + 3, sizeof m_cameraParams.V);
    std::memcpy(m_cameraParams.W, v + 6, sizeof m_cameraParams.W);
    std::memcpy(m_cameraParams.position, v + 9, sizeof m_cameraParams.position);
    // renderersystem.cpp:206: |U| |V| 4 / (width height)
    if (m_backbuffer)
        m_cameraParams.pixelArea =
            len(U) * len(V) * 4.0f / (float)(m_backbuffer->GetWidth() * m_backbuffer->GetHeight());
}

void RendererSystem::SetCamera(const Camera& camera) {
    m_iterationCount = 0;
    m_renderTime = 0;
    m_camera = camera;
    UpdateCameraParams();
    if (m_backbuffer) m_backbuffer->ClearToZero();
    if (m_activeRenderer) m_activeRenderer->SetCamera(camera);
}

void RendererSystem::SetScreenSize(const ei::IVec2& newSize) {
    m_backbuffer.reset();
    m_backbuffer.reset(new DeviceImage(m_ctx, newSize.x, newSize.y));
    m_backbuffer->ClearToZero();
    m_iterationCount = 0;
    m_renderTime = 0;
    UpdateCameraParams();
    if (m_activeRenderer) m_activeRenderer->SetScreenSize(*m_backbuffer);
}

void RendererSystem::Draw() {
    if (!m_activeRenderer) return;
    Check(gpugi_sync(m_ctx));
    const auto begin = std::chrono::steady_clock::now();
    m_activeRenderer->Draw();
    PerIterationBufferUpdate();
    Check(gpugi_sync(m_ctx));
    const auto end = std::chrono::steady_clock::now();
    m_renderTime += (uint64)std::chrono::duration_cast<std::chrono::milliseconds>(end - begin).count();
}

void RendererSystem::SetNumInitialLightSamples(unsigned int numInitialLightSamples) {
    m_numInitialLightSamples = numInitialLightSamples;
    m_lightSamples.assign((size_t)numInitialLightSamples * 8, 0.0f);
    PerIterationBufferUpdate(false);
}

void RendererSystem::ResetIterationCount() { m_iterationCount = 0; }

// renderersystem.cpp:95-116: advance the iteration, draw the next light samples.
void RendererSystem::PerIterationBufferUpdate(bool iterationIncrement) {
    if (iterationIncrement) ++m_iterationCount;
    m_lightSamplerStateBefore = m_lightSamplerState;
    if (m_scene && m_numInitialLightSamples)
        Check(gpugi_generate_light_samples(m_scene->GetHandle(), &m_lightSamplerState, m_numInitialLightSamples,
                                           m_lightSamples.data()));
}

namespace {
// Values of the flat JSON object the checkpoint sidecar is: the text after
// "key": up to the next comma or brace.
bool json_value(const std::string& text, const char* key, std::string& out) {
    const std::string k = std::string("\"") + key + "\"";
    size_t at = text.find(k);
    if (at == std::string::npos) return false;
    at = text.find(':', at + k.size());
    if (at == std::string::npos) return false;
    ++at;
    while (at < text.size() && std::isspace((unsigned char)text[at])) ++at;
    if (at < text.size() && text[at] == '"') {
        const size_t end = text.find('"', at + 1);
        if (end == std::string::npos) return false;
        out = text.substr(at + 1, end - at - 1);
        return true;
    }
    size_t end = at;
    while (end < text.size() && text[end] != ',' && text[end] != '}' && text[end] != '\n') ++end;
    out = text.substr(at, end - at);
    while (!out.empty() && std::isspace((unsigned char)out.back())) out.pop_back();
    return !out.empty();
}

uint64_t json_u64(const std::string& text, const char* key) {
    std::string v;
    if (!json_value(text, key, v)) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, std::string("checkpoint lacks ") + key);
    return std::strtoull(v.c_str(), nullptr, 10);
}

std::string json_escape(const std::string& s) {
    std::string out;
    for (char c : s) {
        if (c == '"' || c == '\\') out += '\\';
        out += c;
    }
    return out;
}

std::string base_name(const std::string& path) {
    const size_t slash = path.find_last_of('/');
    return slash == std::string::npos ? path : path.substr(slash + 1);
}

std::string dir_name(const std::string& path) {
    const size_t slash = path.find_last_of('/');
    return slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
}
}  // namespace

bool RendererSystem::SaveCheckpoint(const std::string& base) const {
    if (!m_backbuffer) return false;
    const int w = m_backbuffer->GetWidth(), h = m_backbuffer->GetHeight();
    const std::vector<float> rgba = m_backbuffer->ReadRGBA();
    if (!WritePfm(rgba.data(), ei::IVec2(w, h), base + ".pfm", (std::uint32_t)m_iterationCount)) return false;
    {
        std::ofstream f((base + ".accum").c_str(), std::ios::binary);
        if (!f) return false;
        f.write(reinterpret_cast<const char*>(rgba.data()), (std::streamsize)(rgba.size() * sizeof(float)));
        if (m_backbuffer->HasFP64()) {
            const std::vector<double> rgb64 = m_backbuffer->ReadRGB64();
            f.write(reinterpret_cast<const char*>(rgb64.data()), (std::streamsize)(rgb64.size() * sizeof(double)));
        }
        if (!f) return false;
    }
    std::ofstream j((base + ".json").c_str());
    if (!j) return false;
    const ei::Vec3 sky = GetSkyRadiance();
    j << "{\n \"format\": \"gpugi_gb300 checkpoint\",\n \"version\": 1,\n"
      << " \"width\": " << w << ",\n \"height\": " << h << ",\n"
      << " \"fp64\": " << (m_backbuffer->HasFP64() ? "true" : "false") << ",\n"
      << " \"iterations\": " << m_iterationCount << ",\n \"next_iteration\": " << m_iterationCount << ",\n"
      << " \"rng_state\": " << m_lightSamplerStateBefore << ",\n"
      << " \"image\": \"" << json_escape(base_name(base)) << ".pfm\",\n"
      << " \"accumulation\": \"" << json_escape(base_name(base)) << ".accum\",\n"
      << " \"renderer\": \"" << json_escape(m_activeRenderer ? m_activeRenderer->GetName() : std::string()) << "\",\n"
      << " \"max_path_length\": " << m_maxPathLength << ",\n \"rr_start_depth\": " << m_rrStartDepth << ",\n"
      << " \"random\": \"" << (m_referenceRng ? "reference" : "pcg") << "\",\n"
      << " \"num_light_samples\": " << m_numInitialLightSamples << ",\n";
    char skyText[96];
    std::snprintf(skyText, sizeof skyText, " \"sky\": [%.9g, %.9g, %.9g]\n}\n", sky.x, sky.y, sky.z);
    j << skyText;
    return (bool)j;
}

void RendererSystem::LoadCheckpoint(const std::string& base) {
    std::ifstream jf((base + ".json").c_str());
    if (!jf) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "cannot read " + base + ".json");
    const std::string text((std::istreambuf_iterator<char>(jf)), std::istreambuf_iterator<char>());
    std::string v;
    if (!json_value(text, "format", v) || v != "gpugi_gb300 checkpoint" || json_u64(text, "version") != 1)
        throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, base + ".json is not a version-1 checkpoint");
    if (!m_backbuffer || (int)json_u64(text, "width") != m_backbuffer->GetWidth() ||
        (int)json_u64(text, "height") != m_backbuffer->GetHeight())
        throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "checkpoint size differs from the screen size");
    if (json_value(text, "renderer", v) && !v.empty() && m_activeRenderer && v != m_activeRenderer->GetName())
        throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "checkpoint of renderer " + v);
    const bool fp64 = json_value(text, "fp64", v) && v == "true";
    std::string accum = base + ".accum";
    if (json_value(text, "accumulation", v)) accum = dir_name(base) + v;
    const size_t n = (size_t)m_backbuffer->GetWidth() * m_backbuffer->GetHeight();
    std::vector<float> rgba(4 * n);
    std::vector<double> rgb64;
    std::ifstream af(accum.c_str(), std::ios::binary);
    af.read(reinterpret_cast<char*>(rgba.data()), (std::streamsize)(rgba.size() * sizeof(float)));
    if (fp64) {
        rgb64.resize(3 * n);
        af.read(reinterpret_cast<char*>(rgb64.data()), (std::streamsize)(rgb64.size() * sizeof(double)));
    }
    if (!af) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "cannot read " + accum);
    if (fp64 && !m_backbuffer->HasFP64()) rgb64.clear();  // the FP32 sums carry the estimate
    m_backbuffer->Write(rgba, rgb64);
    m_iterationCount = (unsigned long)json_u64(text, "next_iteration");
    m_lightSamplerState = json_u64(text, "rng_state");
    PerIterationBufferUpdate(false);  // the light samples of the next iteration
}

gpugi_render_params RendererSystem::MakeRenderParams(gpugi_pass pass) const {
    gpugi_render_params p{};
    p.pass = (uint32_t)pass;
    p.width = (uint32_t)m_backbuffer->GetWidth();
    p.height = (uint32_t)m_backbuffer->GetHeight();
    p.maxPathLength = m_maxPathLength;
    p.rrStartDepth = m_rrStartDepth;
    p.iteration = (uint32_t)m_iterationCount;
    p.samples = 1;
    p.numLightSamples = m_numInitialLightSamples;
    const ei::Vec3 sky = GetSkyRadiance();
    p.sky[0] = sky.x;
    p.sky[1] = sky.y;
    p.sky[2] = sky.z;
    p.flags = m_referenceRng ? GPUGI_RENDER_REFERENCE_RNG : 0u;
    return p;
}

// ------------------------------------------------------------------ Renderers
namespace {
void draw_pass(RendererSystem& sys, gpugi_pass pass) {
    if (!sys.GetScene()) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "no scene set");
    const gpugi_render_params p = sys.MakeRenderParams(pass);
    sys.Check(gpugi_render(sys.GetContext(), sys.GetScene()->GetHandle(), &sys.GetCameraParams(), &p,
                           sys.GetInitialLightSamples(), nullptr, sys.GetBackbuffer().GetHandle()));
}
}  // namespace

// pathtracer.cpp:20-29
Pathtracer::Pathtracer(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(128);
}
void Pathtracer::Draw() { draw_pass(m_rendererSystem, GPUGI_PASS_PT); }

// lightpathtracer.cpp:12-17
LightPathtracer::LightPathtracer(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(256);
}
void LightPathtracer::Draw() { draw_pass(m_rendererSystem, GPUGI_PASS_LT); }

// bidirectionalpathtracer.cpp:20-26
BidirectionalPathtracer::BidirectionalPathtracer(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(128);
}
void BidirectionalPathtracer::Draw() { draw_pass(m_rendererSystem, GPUGI_PASS_BPT); }

WhittedRayTracer::WhittedRayTracer(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(128);  // whittedraytracer.cpp:17
}
void WhittedRayTracer::Draw() { draw_pass(m_rendererSystem, GPUGI_PASS_WHITTED); }

PhotonMapper::PhotonMapper(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(128);  // photonmapper.cpp:38
}
void PhotonMapper::Draw() {
    m_rendererSystem.Check(gpugi_set_photon_config(m_rendererSystem.GetContext(), m_numPhotonsPerLightSample,
                                                   m_queryRadius, m_progressiveRadius ? 1u : 0u));
    draw_pass(m_rendererSystem, GPUGI_PASS_PM);
}

PixelMapLighttracer::PixelMapLighttracer(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(128);  // pixelmaplighttracer.cpp:29
}
void PixelMapLighttracer::Draw() {
    m_rendererSystem.Check(gpugi_set_importon_config(m_rendererSystem.GetContext(), m_numPhotonsPerLightSample,
                                                     m_queryRadius, m_progressiveRadius ? 1u : 0u));
    draw_pass(m_rendererSystem, GPUGI_PASS_IM);
}

// hierarchyimportance.cpp:20-27
HierarchyImportance::HierarchyImportance(RendererSystem& rendererSystem) : Renderer(rendererSystem) {
    m_rendererSystem.SetNumInitialLightSamples(128);
}
// hierarchyimportance.cpp:29-72: the node NDFs and materials of the scene
void HierarchyImportance::SetScene(std::shared_ptr<Scene> scene) {
    if (scene->GetSGGX().empty())
        throw GpugiError(GPUGI_ERROR_INVALID_SCENE, "HierarchyImportance needs the scene's node NDFs (SGGX)");
    m_rendererSystem.Check(
        gpugi_scene_set_hierarchy_ndf(m_rendererSystem.GetContext(), scene->GetHandle(), scene->GetSGGX().data()));
}
// hierarchyimportance.cpp:83-114; MAX_PATHLENGTH 4 (hierarchypathtracer.comp:17)
void HierarchyImportance::Draw() {
    if (!m_rendererSystem.GetScene()) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "no scene set");
    gpugi_render_params p = m_rendererSystem.MakeRenderParams(GPUGI_PASS_HIERARCHY);
    p.maxPathLength = 4;
    m_rendererSystem.Check(gpugi_render(m_rendererSystem.GetContext(), m_rendererSystem.GetScene()->GetHandle(),
                                        &m_rendererSystem.GetCameraParams(), &p,
                                        m_rendererSystem.GetInitialLightSamples(), nullptr,
                                        m_rendererSystem.GetBackbuffer().GetHandle()));
}

NrcPathtracer::NrcPathtracer(RendererSystem& rendererSystem, const NrcSettings& settings)
    : NrcPathtracer(rendererSystem, settings, GPUGI_PASS_PT) {}

NrcPathtracer::NrcPathtracer(RendererSystem& rendererSystem, const NrcSettings& settings, gpugi_pass pass)
    : Renderer(rendererSystem), m_settings(settings), m_pass(pass) {
    m_rendererSystem.SetNumInitialLightSamples(128);  // pathtracer.cpp:28, bidirectionalpathtracer.cpp:25
}

NrcPathtracer::~NrcPathtracer() { gpugi_nrc_destroy(m_nrc); }

void NrcPathtracer::SetScene(std::shared_ptr<Scene> scene) {
    gpugi_nrc_destroy(m_nrc);
    m_nrc = nullptr;
    if (!scene) return;
    ei::Vec3 lo, hi;
    scene->GetBoundingBox(lo, hi);
    const float bmin[3] = {lo.x, lo.y, lo.z}, bmax[3] = {hi.x, hi.y, hi.z};
    m_rendererSystem.Check(gpugi_nrc_create(m_rendererSystem.GetContext(), bmin, bmax, m_settings.seed,
                                            m_settings.learningRate, &m_nrc));
}

void NrcPathtracer::Draw() {
    if (!m_rendererSystem.GetScene() || !m_nrc) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "no scene set");
    const gpugi_render_params p = m_rendererSystem.MakeRenderParams(m_pass);
    gpugi_nrc_params q{};
    q.terminateDepth = m_settings.terminateDepth;
    q.trainFraction = m_settings.trainFraction;
    q.maxTrainSamples = m_settings.maxTrainSamples;
    q.trainSteps = m_settings.trainSteps;
    q.train = m_train ? 1u : 0u;
    m_rendererSystem.Check(gpugi_render_nrc(m_rendererSystem.GetContext(), m_rendererSystem.GetScene()->GetHandle(),
                                            &m_rendererSystem.GetCameraParams(), &p,
                                            m_rendererSystem.GetInitialLightSamples(), nullptr, m_nrc, &q,
                                            m_rendererSystem.GetBackbuffer().GetHandle()));
}

// -------------------------------------------------------------------- imageut
// hdrimage.cpp:6-33: "PF", size, scale -1 (little endian), rows as stored.
bool WritePfm(const float* rgba, const ei::IVec2& size, const std::string& filename, std::uint32_t divisor) {
    std::ofstream file(filename.c_str(), std::ios::binary);
    if (!file) {
        std::fprintf(stderr, "Error writing hdr image to %s\n", filename.c_str());
        return false;
    }
    file.write("PF\n", 3);
    file << size.x << " " << size.y << "\n";
    file.write("-1.000000\n", 10);
    const float d = divisor ? (float)divisor : 1.0f;
    for (int i = 0; i < size.x * size.y; ++i) {
        const float out[3] = {rgba[4 * i] / d, rgba[4 * i + 1] / d, rgba[4 * i + 2] / d};
        file.write(reinterpret_cast<const char*>(out), sizeof out);
    }
    return (bool)file;
}

std::unique_ptr<float[]> LoadPfm(const std::string& filename, ei::IVec2& size) {
    std::ifstream file(filename.c_str(), std::ios::binary);
    if (!file) {
        std::fprintf(stderr, "Error reading hdr image from %s\n", filename.c_str());
        return nullptr;
    }
    char header[3];
    file.read(header, 3);
    if (!file || std::memcmp(header, "PF\n", 3) != 0) return nullptr;
    float scale = 0.0f;
    file >> size.x >> size.y >> scale;
    file.get();  // the single whitespace before the raster
    if (!file || size.x <= 0 || size.y <= 0 || scale >= 0.0f) return nullptr;  // little-endian only
    std::unique_ptr<float[]> out(new float[(size_t)size.x * size.y * 3]);
    file.read(reinterpret_cast<char*>(out.get()), (std::streamsize)((size_t)size.x * size.y * 3 * sizeof(float)));
    if (!file) return nullptr;
    return out;
}

void TextureMSE::LoadReferenceFromPFM(const std::string& filename) {
    auto data = LoadPfm(filename, m_size);
    m_reference.clear();
    if (data) m_reference.assign(data.get(), data.get() + (size_t)m_size.x * m_size.y * 3);
}

// texturemse.cpp:39-65: mean over pixels of the squared RGB error of the
// normalised accumulation; reduced in FP64 (FP64 accumulation when the image has one).
double TextureMSE::ComputeCurrentMSE64(const DeviceImage& texture, unsigned int divisor) {
    if (m_reference.empty()) throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "no reference image loaded");
    if (m_size.x != texture.GetWidth() || m_size.y != texture.GetHeight())
        throw GpugiError(GPUGI_ERROR_INVALID_ARGUMENT, "reference size differs from the image");
    double mse = 0.0;
    check_status(texture.GetContext(),
                 gpugi_image_mse(texture.GetContext(), texture.GetHandle(), (double)(divisor ? divisor : 1),
                                 m_reference.data(), texture.HasFP64() ? 1u : 0u, &mse),
                 "gpugi_image_mse");
    return mse;
}

float TextureMSE::ComputeCurrentMSE(const DeviceImage& texture, unsigned int divisor) {
    return (float)ComputeCurrentMSE64(texture, divisor);
}
