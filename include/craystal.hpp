// craystal.hpp -- C++ facade over the C ABI (craystal_c.h) that keeps the
// class names and call sequence of the reference library's hot path
// (Hyiker/CRaystal, Source/CRaystal/CRaystal.h):
//
//   CRay::SceneData / MeshData / MaterialData   Scene/Scene.h:40-47,
//                                               Scene/Triangle.h:36-42,
//                                               Core/Material.h:34-66
//   CRay::Scene(SceneData&&), setCamera         Scene/Scene.h:50-58
//   CRay::Camera (setters, setSensor)           Core/Camera.h:18-46
//   CRay::Sensor(size, spp), createImage        Core/Sensor.h:33-61
//   CRay::PathTraceIntegrator(Configs).dispatch Core/Integrator.h:10-38
//   CRay::Image (load, writeEXR, writePNG)      Utils/Image.h:24-90
//   CRay::Importer().import(xml)                Utils/Importer.h:10-28
//
// Header-only; link with libcraystal_gb300.so.  Errors throw
// CRay::RuntimeError, as the reference's CRAYSTAL_CHECK does.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "craystal_c.h"

namespace CRay {

using Float = float;
struct Float2 {
    float x = 0, y = 0;
};
struct Float3 {
    float x = 0, y = 0, z = 0;
};
struct UInt2 {
    uint32_t x = 0, y = 0;
};

class RuntimeError : public std::runtime_error {
   public:
    explicit RuntimeError(const std::string& m) : std::runtime_error(m) {}
};

inline void crCheck(int code) {
    if (code != CR_OK) throw RuntimeError(std::string("craystal_gb300: ") + cr_last_error());
}

enum class MaterialType : uint32_t { FullDiffuse = 0, Principled = 1, Phong = 2 };
enum class MaterialFlags : uint32_t { IsEmissive = 1, IsDiffuse = 2, hasDiffuseTexture = 4 };

/** Utils/Image.h:24-90: float pixels, interleaved (y * width + x) * channels + c. */
class Image {
   public:
    using Ref = std::shared_ptr<Image>;
    Image(size_t width, size_t height, int channels)
        : mWidth(uint32_t(width)), mHeight(uint32_t(height)), mChannels(uint32_t(channels)),
          mData(width * height * size_t(channels), 0.0f) {}
    int getWidth() const { return int(mWidth); }
    int getHeight() const { return int(mHeight); }
    int getChannels() const { return int(mChannels); }
    int getArea() const { return int(mWidth * mHeight); }
    float getPixel(int x, int y, int c) const { return mData[(size_t(y) * mWidth + x) * mChannels + c]; }
    void setPixel(int x, int y, int c, float v) { mData[(size_t(y) * mWidth + x) * mChannels + c] = v; }
    std::vector<float>& data() { return mData; }
    const std::vector<float>& data() const { return mData; }
    /** Image::writeEXR, Utils/Image.cpp:49-106. */
    void writeEXR(const std::string& path) const {
        crCheck(cr_image_write_exr(path.c_str(), mWidth, mHeight, mChannels, mData.data()));
    }
    /** Image::writePNG, Utils/Image.cpp:182-217. */
    void writePNG(const std::string& path, bool gammaCorrect) const {
        crCheck(cr_image_write_png(path.c_str(), mWidth, mHeight, mChannels, mData.data(), gammaCorrect ? 1 : 0));
    }
    /** Image::load, Utils/Image.cpp:262-270. */
    static Image load(const std::string& path, bool toLinear = true) {
        cr_image img{};
        crCheck(cr_image_load(path.c_str(), toLinear ? 1 : 0, &img));
        Image out(img.width, img.height, int(img.channels));
        std::copy(img.pixels, img.pixels + out.mData.size(), out.mData.begin());
        cr_image_free(&img);
        return out;
    }

   private:
    uint32_t mWidth, mHeight, mChannels;
    std::vector<float> mData;
};

struct MaterialData {
    Float3 diffuseRefl;
    Float3 specularRefl;
    Float3 emission;
    Float shininess = 0;
    MaterialType type = MaterialType::FullDiffuse;
    uint32_t flags = 0;
    uint32_t diffuseHandle = 0;  ///< texture index when flags has hasDiffuseTexture

    bool isEmissive() const { return flags & uint32_t(MaterialFlags::IsEmissive); }
    // MaterialData::finalize, Core/Material.h:57-65
    void finalize() {
        auto mx = [](Float3 v) { return std::max(std::max(v.x, v.y), v.z); };
        if (mx(emission) != 0.0f) flags |= uint32_t(MaterialFlags::IsEmissive);
        if (mx(specularRefl) == 0.0f) flags |= uint32_t(MaterialFlags::IsDiffuse);
    }
};

struct MeshData {
    std::vector<Float3> position;
    std::vector<Float3> normal;
    std::vector<Float2> texCrd;
    std::vector<uint32_t> index;
    uint32_t materialID = 0;
};

struct SceneData {
    std::vector<MeshData> meshes;
    std::vector<MaterialData> materials;
    std::vector<uint32_t> emissiveIndex;
    std::vector<Image> textureImages;
};

/** Film of a sensor; the host copy is filled by PathTraceIntegrator::dispatch. */
class Sensor {
   public:
    using Ref = std::shared_ptr<Sensor>;
    explicit Sensor(UInt2 size, uint32_t spp = 1u) : mSize(size), mSpp(spp) {
        mData.assign(size_t(size.x) * size.y * 3, 0.0f);
        mWeight.assign(size_t(size.x) * size.y, 0.0f);
    }
    void setSPP(uint32_t v) { mSpp = v; }
    uint32_t getSPP() const { return mSpp; }
    UInt2 getSize() const { return mSize; }
    /** Sensor::createImage (Core/Sensor.cu:93-112): rgb = sum / weight, row-major, 3 floats per pixel. */
    Image::Ref createImage() const {
        auto img = std::make_shared<Image>(mSize.x, mSize.y, 3);
        for (size_t i = 0; i < mWeight.size(); i++)
            for (int c = 0; c < 3; c++) img->data()[3 * i + c] = mData[3 * i + c] / mWeight[i];
        return img;
    }
    std::vector<float>& data() { return mData; }
    std::vector<float>& weight() { return mWeight; }

   private:
    UInt2 mSize;
    uint32_t mSpp;
    std::vector<float> mData, mWeight;
};

class Camera {
   public:
    using Ref = std::shared_ptr<Camera>;
    void setFovY(Float v) { mFovY = v; }
    void setWorldPosition(const Float3& p) { mPos = p; }
    void setTarget(const Float3& t) { mTarget = t; }
    void setUp(const Float3& u) { mUp = u; }
    void setSensor(const Sensor::Ref& s) { mSensor = s; }
    Sensor::Ref getSensor() { return mSensor; }
    /** The basis is computed by the library when the camera is set on a scene. */
    void calculateCameraData() const {}

    cr_camera toC() const {
        cr_camera c{};
        c.pos[0] = mPos.x, c.pos[1] = mPos.y, c.pos[2] = mPos.z;
        c.target[0] = mTarget.x, c.target[1] = mTarget.y, c.target[2] = mTarget.z;
        c.up[0] = mUp.x, c.up[1] = mUp.y, c.up[2] = mUp.z;
        c.fov_y = mFovY;
        c.width = mSensor ? mSensor->getSize().x : 512u;
        c.height = mSensor ? mSensor->getSize().y : 512u;
        return c;
    }

   private:
    // CameraProxy defaults, Core/CameraProxy.h:12-23
    Float3 mPos{0, 0, 0};
    Float mFovY = 60.f;
    Float3 mTarget{0, 0, -1};
    Float3 mUp{0, 1, 0};
    Sensor::Ref mSensor;
};

class Importer;

class Scene {
   public:
    using Ref = std::shared_ptr<Scene>;
    /** Scene(SceneData&&), Scene/Scene.cu:61-78: uploads and builds the BVH on the GPU. */
    explicit Scene(SceneData&& data) {
        std::vector<float> pos, nrm, uv;
        std::vector<uint32_t> idx;
        std::vector<cr_mesh_desc> descs;
        for (const MeshData& m : data.meshes) {
            cr_mesh_desc d{};
            d.index_offset = uint32_t(idx.size());
            d.index_count = uint32_t(m.index.size());
            d.vertex_offset = uint32_t(pos.size() / 3);
            d.material_id = m.materialID;
            for (size_t i = 0; i < m.position.size(); i++) {
                pos.insert(pos.end(), {m.position[i].x, m.position[i].y, m.position[i].z});
                Float3 n = i < m.normal.size() ? m.normal[i] : Float3{};
                nrm.insert(nrm.end(), {n.x, n.y, n.z});
                Float2 t = i < m.texCrd.size() ? m.texCrd[i] : Float2{};
                uv.insert(uv.end(), {t.x, t.y});
            }
            for (uint32_t v : m.index) idx.push_back(v + d.vertex_offset);
            descs.push_back(d);
        }
        std::vector<cr_material> mats;
        for (const MaterialData& md : data.materials) {
            cr_material c{};
            c.diffuse[0] = md.diffuseRefl.x, c.diffuse[1] = md.diffuseRefl.y, c.diffuse[2] = md.diffuseRefl.z;
            c.specular[0] = md.specularRefl.x, c.specular[1] = md.specularRefl.y, c.specular[2] = md.specularRefl.z;
            c.emission[0] = md.emission.x, c.emission[1] = md.emission.y, c.emission[2] = md.emission.z;
            c.shininess = md.shininess;
            c.type = uint32_t(md.type);
            c.flags = md.flags;
            mats.push_back(c);
        }
        cr_scene* s = nullptr;
        crCheck(cr_scene_create(pos.data(), nrm.data(), uv.data(), pos.size() / 3, idx.data(), idx.size() / 3,
                                descs.data(), uint32_t(descs.size()), mats.data(), uint32_t(mats.size()),
                                data.emissiveIndex.data(), uint32_t(data.emissiveIndex.size()), &s));
        mScene.reset(s, [](cr_scene* p) { cr_scene_destroy(p); });
        if (!data.textureImages.empty()) {
            // Texture(const Image&), Core/Texture.cu:45-60: RGBA texels, missing channels 0
            std::vector<std::vector<float>> texels;
            std::vector<cr_texture> texs;
            for (const Image& im : data.textureImages) {
                std::vector<float> t(size_t(im.getArea()) * 4, 0.0f);
                for (int p = 0; p < im.getArea(); p++)
                    for (int c = 0; c < std::min(im.getChannels(), 4); c++)
                        t[4 * size_t(p) + c] = im.data()[size_t(p) * im.getChannels() + c];
                texels.push_back(std::move(t));
            }
            for (size_t i = 0; i < texels.size(); i++)
                texs.push_back(cr_texture{uint32_t(data.textureImages[i].getWidth()),
                                          uint32_t(data.textureImages[i].getHeight()), texels[i].data()});
            std::vector<uint32_t> matTex;
            for (const MaterialData& md : data.materials)
                matTex.push_back(md.flags & uint32_t(MaterialFlags::hasDiffuseTexture) ? md.diffuseHandle
                                                                                       : CR_NO_TEXTURE);
            crCheck(cr_scene_set_diffuse_textures(s, texs.data(), uint32_t(texs.size()), matTex.data(),
                                                  uint32_t(matTex.size())));
        }
    }
    Camera::Ref getCamera() { return mCamera; }
    void setCamera(const Camera::Ref& c) {
        mCamera = c;
        cr_camera cc = c->toC();
        crCheck(cr_scene_set_camera(mScene.get(), &cc));
    }
    cr_scene* handle() const { return mScene.get(); }

   private:
    friend class Importer;
    explicit Scene(cr_scene* s) { mScene.reset(s, [](cr_scene* p) { cr_scene_destroy(p); }); }
    std::shared_ptr<cr_scene> mScene;
    Camera::Ref mCamera;
};

/** Utils/Importer.h:10-28: an XML scene description beside an OBJ/MTL file
 *  of the same name. */
class Importer {
   public:
    /** Importer::import (Utils/Importer.cpp:203-236): the scene with its camera set. */
    Scene::Ref import(const std::string& path) {
        cr_import* imp = nullptr;
        crCheck(cr_import_xml(path.c_str(), &imp));
        std::unique_ptr<cr_import, int (*)(cr_import*)> guard(imp, cr_import_destroy);
        cr_import_view v{};
        crCheck(cr_import_get(imp, &v));
        cr_scene* s = nullptr;
        crCheck(cr_import_create_scene(imp, &s));
        Scene::Ref scene(new Scene(s));
        auto cam = std::make_shared<Camera>();
        cam->setWorldPosition({v.camera.pos[0], v.camera.pos[1], v.camera.pos[2]});
        cam->setTarget({v.camera.target[0], v.camera.target[1], v.camera.target[2]});
        cam->setUp({v.camera.up[0], v.camera.up[1], v.camera.up[2]});
        cam->setFovY(v.camera.fov_y);
        cam->setSensor(std::make_shared<Sensor>(UInt2{v.camera.width, v.camera.height}));
        scene->setCamera(cam);
        return scene;
    }
};

class PathTraceIntegrator {
   public:
    using Ref = std::shared_ptr<PathTraceIntegrator>;
    struct Configs {
        uint32_t maxDepth = 10u;
        Float rrThreshold = 0.15f;
        bool useMIS = true;
    };
    /** compat = true keeps the reference's effective device values
     *  (maxDepth 10, rrThreshold 0.05, Core/Integrator.h:20-23): its
     *  Configs are never copied to the device. */
    explicit PathTraceIntegrator(Configs c, bool compat = true) : mConfigs(c), mCompat(compat) {}

    /** PathTraceIntegrator::dispatch, Core/Integrator.cu:233-262. */
    void dispatch(Scene& scene, int spp, uint32_t firstSample = 0) const {
        auto cam = scene.getCamera();
        if (!cam || !cam->getSensor()) throw RuntimeError("scene has no camera with a sensor");
        auto sensor = cam->getSensor();
        sensor->setSPP(uint32_t(spp));
        scene.setCamera(cam);
        cr_integrator_config cfg{};
        cfg.max_depth = mCompat ? 10u : mConfigs.maxDepth;
        cfg.rr_threshold = mCompat ? 0.05f : mConfigs.rrThreshold;
        cfg.use_mis = mConfigs.useMIS ? 1u : 0u;
        crCheck(cr_render(scene.handle(), &cfg, uint32_t(spp), firstSample, nullptr));
        crCheck(cr_film_read(scene.handle(), sensor->data().data(), sensor->weight().data()));
    }

   private:
    Configs mConfigs;
    bool mCompat;
};

}  // namespace CRay
