// cr_method.hpp -- C++ adapter with the shape of the reference's Method
// plugin, over the C ABI of cr_raster.h (header only).
//
// The reference's plugin interface is `struct Method { string name,
// description, group; virtual void update(Renderer*) = 0; virtual void
// render(Renderer*) = 0; }` (include/Method.h:10-24), registered with
// Runtime::addMethod and selected by name (include/Runtime.h:37-49), and
// called once per frame for Renderer::views[0] (src/main.cpp:342, :455;
// include/Renderer.h:78-82).  Here the Renderer is replaced by the one thing
// these methods read from it -- the view's matrices and framebuffer size --
// and the image stays in device memory (CR_FB_IMAGE) for the caller to
// display or copy.
//
//   cr::RasterMethod m(ctx, "loop_las");   // name/group/description as registered
//   m.set_cloud(cloud);
//   m.update();                            // no-op, as for the reference's methods
//   m.render(target, stream);              // cull + raster + resolve (+ re-clear)
//   m.read_image(host, stream);            // or m.image_device()
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cr_raster.h"

namespace cr {

// What a method reads from Renderer::views[0] (Renderer.h:78-82): column-major
// view and projection matrices (glm layout, double) and the framebuffer size.
struct ViewTarget {
    double view[16];
    double proj[16];
    int32_t width = 0;
    int32_t height = 0;
};

// The reference's Method (include/Method.h:10-24) without the Renderer.
class Method {
  public:
    std::string name = "no name";
    std::string description;
    std::string group = "no group";
    virtual ~Method() = default;
    virtual void update() = 0;
    virtual void render(const ViewTarget& target, void* stream) = 0;
};

// Registered name, group and description of a method, without a context.
inline bool method_info(const char* method_name, int32_t* id, std::string* name,
                        std::string* group, std::string* description) {
    int32_t m = 0;
    if (cr_method_find(method_name, &m) != CR_OK) return false;
    if (id) *id = m;
    if (name) *name = cr_method_name(m);
    if (group) *group = cr_method_group(m);
    if (description) *description = cr_method_description(m);
    return true;
}

// "loop_las", "loop_las_prefetch", "loop_las_hqs" (LAS-derived clouds) or
// "(2021) early-z" (plain 16 B clouds), rendered through cr_render.  The
// framebuffer is created on the first frame and recreated when the target
// size changes, as the reference's methods resize theirs
// (compute_loop_las.h:130-138).  Errors do not throw from render(): like the
// reference, a failed frame leaves the previous image; last_status() and
// last_error() report it.
class RasterMethod : public Method {
  public:
    RasterMethod(cr_ctx* ctx, const char* method_name) : ctx_(ctx) {
        if (!ctx_ || !method_info(method_name, &id_, &name, &group, &description))
            throw std::invalid_argument(std::string("unknown method: ") + method_name);
        cr_render_params_default(id_, &params_);
        params_.resolve = 1;
        params_.clear_after = 1;
    }
    RasterMethod(const RasterMethod&) = delete;
    RasterMethod& operator=(const RasterMethod&) = delete;
    ~RasterMethod() override {
        if (fb_) cr_fb_destroy(ctx_, fb_);
    }

    void set_cloud(const cr_cloud* cloud) { cloud_ = cloud; }
    cr_render_params& params() { return params_; }
    int32_t method_id() const { return id_; }

    void update() override {}

    void render(const ViewTarget& t, void* stream) override {
        status_ = frame(t, stream);
    }

    cr_status last_status() const { return status_; }
    std::string last_error() const { return cr_last_error(ctx_); }
    cr_fb* framebuffer() const { return fb_; }

    // Device address of the RGBA8 image (width * height u32), or nullptr.
    const uint32_t* image_device() const {
        void* p = nullptr;
        if (!fb_ || cr_fb_device(fb_, CR_FB_IMAGE, &p) != CR_OK) return nullptr;
        return static_cast<const uint32_t*>(p);
    }

    // Copies the image to host memory (width * height u32) on `stream`.
    cr_status read_image(uint32_t* host, void* stream) const {
        if (!fb_) return CR_ERR_INVALID_ARG;
        return cr_fb_read(ctx_, fb_, CR_FB_IMAGE, host, (int64_t)w_ * h_ * 4, stream);
    }

  private:
    cr_status frame(const ViewTarget& t, void* stream) {
        if (!cloud_) return CR_ERR_INVALID_ARG;
        if (!fb_ || t.width != w_ || t.height != h_) {
            if (fb_) cr_fb_destroy(ctx_, fb_);
            fb_ = nullptr;
            const int32_t kind = id_ == CR_METHOD_LOOP_LAS_HQS ? CR_FB_HQS : CR_FB_U64;
            cr_status s = cr_fb_create(ctx_, t.width, t.height, kind, &fb_);
            if (s != CR_OK) return s;
            w_ = t.width;
            h_ = t.height;
            // HQS depth starts at -inf bits (compute_loop_las_hqs.h:336-340)
            s = cr_fb_clear(ctx_, fb_, kind == CR_FB_HQS ? 0xFF800000ull : params_.clear_value, stream);
            if (s != CR_OK) return s;
        }
        cr_view v;
        std::memcpy(v.view, t.view, sizeof(v.view));
        std::memcpy(v.proj, t.proj, sizeof(v.proj));
        v.width = t.width;
        v.height = t.height;
        return cr_render(ctx_, cloud_, &v, &params_, fb_, stream);
    }

    cr_ctx* ctx_ = nullptr;
    const cr_cloud* cloud_ = nullptr;
    cr_fb* fb_ = nullptr;
    int32_t id_ = 0;
    int32_t w_ = 0, h_ = 0;
    cr_render_params params_{};
    cr_status status_ = CR_OK;
};

// The reference's Runtime method list (include/Runtime.h:37-49): methods are
// added once and one is selected by name.
class MethodRegistry {
  public:
    Method* add(std::unique_ptr<Method> m) {
        methods_.push_back(std::move(m));
        if (!selected_) selected_ = methods_.back().get();
        return methods_.back().get();
    }
    Method* select(const std::string& name) {
        for (auto& m : methods_)
            if (m->name == name) return selected_ = m.get();
        return nullptr;
    }
    Method* selected() const { return selected_; }
    const std::vector<std::unique_ptr<Method>>& methods() const { return methods_; }

  private:
    std::vector<std::unique_ptr<Method>> methods_;
    Method* selected_ = nullptr;
};

}  // namespace cr
