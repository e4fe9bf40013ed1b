// crayli_demo.cpp -- the reference's CRayli flow (Source/CRayli/CRayli.cpp:
// build a scene, set a camera with a sensor, PathTraceIntegrator::dispatch,
// Sensor::createImage) written against the C++ facade craystal.hpp.
// Scene: a floor quad and a ceiling light quad; writes the resolved image as
// raw float32 (width, height, 3) to the path given as argv[1].
#include <cstdio>
#include <vector>

#include "craystal.hpp"

int main(int argc, char** argv) {
    using namespace CRay;
    SceneData data;
    MeshData floor;
    floor.position = {{-1, -1, -1}, {1, -1, -1}, {1, -1, 1}, {-1, -1, 1}};
    floor.normal = {{0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 1, 0}};
    floor.index = {0, 2, 1, 0, 3, 2};
    floor.materialID = 0;
    MeshData light;
    light.position = {{-0.3f, 0.9f, -0.3f}, {0.3f, 0.9f, -0.3f}, {0.3f, 0.9f, 0.3f}, {-0.3f, 0.9f, 0.3f}};
    light.normal = {{0, -1, 0}, {0, -1, 0}, {0, -1, 0}, {0, -1, 0}};
    light.index = {0, 1, 2, 0, 2, 3};
    light.materialID = 1;
    data.meshes = {floor, light};
    MaterialData diffuse;
    diffuse.diffuseRefl = {0.7f, 0.5f, 0.3f};
    diffuse.type = MaterialType::Phong;
    diffuse.specularRefl = {0.1f, 0.1f, 0.1f};
    diffuse.shininess = 16.0f;
    diffuse.finalize();
    MaterialData emitter;
    emitter.emission = {10, 10, 10};
    emitter.finalize();
    data.materials = {diffuse, emitter};
    data.emissiveIndex = {2, 3};
    try {
        Scene scene(std::move(data));
        auto cam = std::make_shared<Camera>();
        cam->setWorldPosition({0, 0.2f, 3});
        cam->setTarget({0, -0.5f, 0});
        cam->setUp({0, 1, 0});
        cam->setFovY(45);
        auto sensor = std::make_shared<Sensor>(UInt2{64, 48});
        cam->setSensor(sensor);
        scene.setCamera(cam);
        PathTraceIntegrator integ(PathTraceIntegrator::Configs{});
        integ.dispatch(scene, 8);
        const std::vector<float>& img = sensor->createImage()->data();
        if (argc > 1) {
            FILE* f = std::fopen(argv[1], "wb");
            if (!f) return 2;
            std::fwrite(img.data(), sizeof(float), img.size(), f);
            std::fclose(f);
        }
        double sum = 0;
        for (float v : img) sum += v == v ? v : 0.0;
        std::printf("crayli_demo: %ux%u, mean %.6f\n", sensor->getSize().x, sensor->getSize().y, sum / img.size());
    } catch (const RuntimeError& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
