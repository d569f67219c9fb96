// Headless front end of the C++ renderer classes: loads a scene file, sets
// up a RendererSystem like Application does (application.cpp:211-260,
// 346-376) and draws a number of iterations, then writes the normalised
// backbuffer as PFM (Application::SaveImage) and prints a JSON summary.
//
//   gpugi_headless --scene FILE [--renderer Pathtracer|LightPathtracer|
//                  BidirectionalPathtracer|NrcPathtracer|
//                  NrcBidirectionalPathtracer|WhittedRayTracer|PhotonMapper|
//                  PixelMapLighttracer|HierarchyImportance]
//                  [--size W H]
//                  [--camera px py pz lx ly lz fovy] [--iterations N]
//                  [--path-length L] [--rr-start D] [--sky r g b] [--reference-rng]
//                  [--point-light px py pz ir ig ib] [--reference FILE.pfm]
//                  [--out FILE.pfm] [--checkpoint BASE] [--resume BASE] [--device D]
//                  [--mse-check-interval N] [--wait-mse X]
//
// --mse-check-interval N computes the MSE against --reference every N
// iterations and prints it as a JSON line (Application::MSEChecks,
// application.cpp:345-376, the GlobalConfig `mseCheckInterval`);
// --wait-mse X stops drawing at the first check whose MSE is below X, or
// whose MSE is NaN (the script command `waitMSE`), with --iterations as the
// cap. The summary line then says whether X was reached and when.
// --resume BASE restores a checkpoint (RendererSystem::LoadCheckpoint) before
// drawing, --checkpoint BASE writes one after (SaveCheckpoint), so a long
// accumulation can run as several invocations with the same settings.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gpugi_renderer.hpp"

namespace {

struct Args {
    std::string scene, renderer = "Pathtracer", out, reference, checkpoint, resume;
    int width = 256, height = 256, iterations = 16, device = 0, mseCheckInterval = 0;
    double waitMse = 0.0;
    unsigned pathLength = 8, rrStart = 0;
    float cam[7] = {0.0f, 1.0f, 3.4f, 0.0f, 1.0f, 0.0f, 40.0f};
    float sky[3] = {0.0f, 0.0f, 0.0f};
    bool referenceRng = false;
    std::vector<PointLight> pointLights;
};

[[noreturn]] void usage(const char* msg) {
    std::fprintf(stderr, "gpugi_headless: %s\n", msg);
    std::exit(2);
}

Args parse(int argc, char** argv) {
    Args a;
    auto need = [&](int& i, int n) {
        if (i + n >= argc) usage((std::string("missing values after ") + argv[i]).c_str());
    };
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        if (k == "--scene") { need(i, 1); a.scene = argv[++i]; }
        else if (k == "--renderer") { need(i, 1); a.renderer = argv[++i]; }
        else if (k == "--out") { need(i, 1); a.out = argv[++i]; }
        else if (k == "--reference") { need(i, 1); a.reference = argv[++i]; }
        else if (k == "--checkpoint") { need(i, 1); a.checkpoint = argv[++i]; }
        else if (k == "--resume") { need(i, 1); a.resume = argv[++i]; }
        else if (k == "--size") { need(i, 2); a.width = std::atoi(argv[++i]); a.height = std::atoi(argv[++i]); }
        else if (k == "--iterations") { need(i, 1); a.iterations = std::atoi(argv[++i]); }
        else if (k == "--device") { need(i, 1); a.device = std::atoi(argv[++i]); }
        else if (k == "--mse-check-interval") { need(i, 1); a.mseCheckInterval = std::atoi(argv[++i]); }
        else if (k == "--wait-mse") { need(i, 1); a.waitMse = std::strtod(argv[++i], nullptr); }
        else if (k == "--path-length") { need(i, 1); a.pathLength = (unsigned)std::atoi(argv[++i]); }
        else if (k == "--rr-start") { need(i, 1); a.rrStart = (unsigned)std::atoi(argv[++i]); }
        else if (k == "--reference-rng") { a.referenceRng = true; }
        else if (k == "--camera") { need(i, 7); for (float& c : a.cam) c = std::strtof(argv[++i], nullptr); }
        else if (k == "--sky") { need(i, 3); for (float& c : a.sky) c = std::strtof(argv[++i], nullptr); }
        else if (k == "--point-light") {
            need(i, 6);
            PointLight p;
            p.position = ei::Vec3(std::strtof(argv[i + 1], nullptr), std::strtof(argv[i + 2], nullptr),
                                  std::strtof(argv[i + 3], nullptr));
            p.intensity = ei::Vec3(std::strtof(argv[i + 4], nullptr), std::strtof(argv[i + 5], nullptr),
                                   std::strtof(argv[i + 6], nullptr));
            a.pointLights.push_back(p);
            i += 6;
        } else usage((std::string("unknown argument ") + k).c_str());
    }
    if (a.scene.empty()) usage("--scene is required");
    if (a.width <= 0 || a.height <= 0 || a.iterations < 0) usage("bad size or iteration count");
    if (a.mseCheckInterval < 0) usage("--mse-check-interval must be >= 0");
    if (a.mseCheckInterval > 0 && a.reference.empty()) usage("--mse-check-interval needs --reference");
    // the reference refuses waitMSE without an MSE check interval or a reference image
    if (a.waitMse > 0.0 && a.mseCheckInterval <= 0) usage("--wait-mse needs --mse-check-interval > 0");
    return a;
}

}  // namespace

int main(int argc, char** argv) {
    const Args a = parse(argc, argv);
    try {
        RendererSystem system(a.device);
        system.SetScreenSize(ei::IVec2(a.width, a.height));
        system.SetMaxPathLength(a.pathLength);
        system.SetRussianRouletteStart(a.rrStart);
        system.SetReferenceRandomStreams(a.referenceRng);
        auto scene = std::make_shared<Scene>(system.GetContext(), a.scene);
        for (const PointLight& p : a.pointLights) scene->AddPointLight(p);
        system.SetScene(scene);
        system.SetCamera(Camera(ei::Vec3(a.cam[0], a.cam[1], a.cam[2]), ei::Vec3(a.cam[3], a.cam[4], a.cam[5]),
                                (float)a.width / (float)a.height, a.cam[6]));
        auto env = std::make_shared<Environment>();
        env->radiance = ei::Vec3(a.sky[0], a.sky[1], a.sky[2]);
        system.SetEnvironmentMap(env);
        if (a.renderer == "Pathtracer") system.SetRenderer<Pathtracer>();
        else if (a.renderer == "LightPathtracer") system.SetRenderer<LightPathtracer>();
        else if (a.renderer == "BidirectionalPathtracer") system.SetRenderer<BidirectionalPathtracer>();
        else if (a.renderer == "NrcPathtracer") system.SetRenderer<NrcPathtracer>();
        else if (a.renderer == "NrcBidirectionalPathtracer") system.SetRenderer<NrcBidirectionalPathtracer>();
        else if (a.renderer == "WhittedRayTracer") system.SetRenderer<WhittedRayTracer>();
        else if (a.renderer == "PhotonMapper") system.SetRenderer<PhotonMapper>();
        else if (a.renderer == "PixelMapLighttracer") system.SetRenderer<PixelMapLighttracer>();
        else if (a.renderer == "HierarchyImportance") system.SetRenderer<HierarchyImportance>();
        else usage("unknown renderer");

        if (!a.resume.empty()) system.LoadCheckpoint(a.resume);
        TextureMSE tmse;
        if (!a.reference.empty()) {
            tmse.LoadReferenceFromPFM(a.reference);
            if (!tmse.HasValidReferenceImage()) usage("cannot read the reference image");
        }
        // Draw, with the MSE checks of Application::MSEChecks every
        // mseCheckInterval iterations; waitMSE ends the loop once the MSE is
        // below the goal (or NaN).
        const auto t0 = std::chrono::steady_clock::now();
        auto wallMs = [&] {
            return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        };
        bool waiting = a.waitMse > 0.0, reached = false, nanMse = false;
        double reachedWallMs = -1.0;
        unsigned long reachedIteration = 0;
        int sinceCheck = 0;
        for (int i = 0; i < a.iterations && !(a.waitMse > 0.0 && !waiting); ++i) {
            system.Draw();
            if (a.mseCheckInterval > 0 && ++sinceCheck >= a.mseCheckInterval) {
                sinceCheck = 0;
                const unsigned long it = system.GetIterationCount();
                const double m = tmse.ComputeCurrentMSE64(system.GetBackbuffer(), (unsigned)it);
                std::printf("{\"iteration\": %lu, \"render_ms\": %llu, \"wall_ms\": %.3f, \"mse\": %.9g}\n", it,
                            (unsigned long long)system.GetRenderTime(), wallMs(), m);
                if (waiting && (m != m || a.waitMse > m)) {
                    waiting = false;
                    nanMse = m != m;
                    reached = !nanMse;
                    reachedWallMs = wallMs();
                    reachedIteration = it;
                }
            }
        }
        std::fflush(stdout);
        if (!a.checkpoint.empty() && !system.SaveCheckpoint(a.checkpoint)) usage("cannot write the checkpoint");

        const unsigned long iterations = system.GetIterationCount();
        double mse = -1.0;
        if (!a.reference.empty()) mse = tmse.ComputeCurrentMSE64(system.GetBackbuffer(), (unsigned)iterations);
        if (!a.out.empty()) {
            const std::vector<float> rgba = system.GetBackbuffer().ReadRGBA();
            if (!WritePfm(rgba.data(), ei::IVec2(a.width, a.height), a.out, (std::uint32_t)iterations)) return 1;
        }
        std::printf(
            "{\"renderer\": \"%s\", \"iterations\": %lu, \"render_ms\": %llu, \"width\": %d, \"height\": %d, "
            "\"mse\": %.9g",
            system.GetActiveRenderer()->GetName().c_str(), iterations, (unsigned long long)system.GetRenderTime(),
            a.width, a.height, mse);
        if (a.waitMse > 0.0)
            std::printf(", \"wait_mse\": %.9g, \"reached\": %s, \"mse_nan\": %s, \"reached_iteration\": %lu, "
                        "\"reached_wall_ms\": %.3f",
                        a.waitMse, reached ? "true" : "false", nanMse ? "true" : "false", reachedIteration,
                        reachedWallMs);
        std::printf("}\n");
        scene.reset();
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "gpugi_headless: %s\n", e.what());
        return 1;
    }
}
