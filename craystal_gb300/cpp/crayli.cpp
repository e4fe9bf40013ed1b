// crayli.cpp -- the reference's command-line renderer (Source/CRayli/
// CRayli.cpp:16-42) on the C++ facade: import an XML + OBJ scene, render
// spp samples per pixel with the path tracer (MIS unless --no-mis), write
// the film as an EXR image.
//
//   crayli <model.xml> [--spp N] [--no-mis] [--out craystal.exr]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "craystal.hpp"

int main(int argc, char** argv) {
    using namespace CRay;
    std::string model, out = "craystal.exr";
    int spp = 16;
    bool noMIS = false;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--spp") && i + 1 < argc) {
            spp = std::atoi(argv[++i]);
        } else if (!std::strcmp(argv[i], "--no-mis")) {
            noMIS = true;
        } else if (!std::strcmp(argv[i], "--out") && i + 1 < argc) {
            out = argv[++i];
        } else if (argv[i][0] != '-' && model.empty()) {
            model = argv[i];
        } else {
            std::fprintf(stderr, "usage: crayli <model.xml> [--spp N] [--no-mis] [--out file.exr]\n");
            return 2;
        }
    }
    if (model.empty() || spp <= 0) {
        std::fprintf(stderr, "usage: crayli <model.xml> [--spp N] [--no-mis] [--out file.exr]\n");
        return 2;
    }
    try {
        Importer importer;
        auto scene = importer.import(model);
        PathTraceIntegrator::Configs conf;
        conf.useMIS = !noMIS;
        PathTraceIntegrator integrator(conf);
        integrator.dispatch(*scene, spp);
        scene->getCamera()->getSensor()->createImage()->writeEXR(out);
        std::printf("crayli: wrote %s (%d spp)\n", out.c_str(), spp);
    } catch (const RuntimeError& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
