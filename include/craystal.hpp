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
enum class MaterialFlags : uint32_t { IsEmissive = 1, IsDiffuse = 2 };

struct MaterialData {
    Float3 diffuseRefl;
    Float3 specularRefl;
    Float3 emission;
    Float shininess = 0;
    MaterialType type = MaterialType::FullDiffuse;
    uint32_t flags = 0;

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
    std::vector<float> createImage() const {
        std::vector<float> img(mData.size());
        for (size_t i = 0; i < mWeight.size(); i++)
            for (int c = 0; c < 3; c++) img[3 * i + c] = mData[3 * i + c] / mWeight[i];
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
    }
    Camera::Ref getCamera() { return mCamera; }
    void setCamera(const Camera::Ref& c) {
        mCamera = c;
        cr_camera cc = c->toC();
        crCheck(cr_scene_set_camera(mScene.get(), &cc));
    }
    cr_scene* handle() const { return mScene.get(); }

   private:
    std::shared_ptr<cr_scene> mScene;
    Camera::Ref mCamera;
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
