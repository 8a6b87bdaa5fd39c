// glm_probe.cpp -- builds the reference's own matrix code path against the
// glm headers vendored in the reference tree (libs/glm, header-only), so the
// CPU tests can pin the oracle's and the product's host matrix setup to it.
// TEST INFRASTRUCTURE: compiled by oracle/Makefile into oracle/_ref/ only when
// the reference tree is present.  Each function evaluates the same glm
// expressions as the reference file:line it names.
#include <cstring>
#include "glm/common.hpp"
#include "glm/matrix.hpp"
#include <glm/gtx/transform.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <glm/gtc/type_ptr.hpp>

using glm::dmat4;
using glm::dvec3;
using glm::mat4;

extern "C" {

// Camera.h:34-39
void glmref_camera(double fovy_deg, int width, int height, double znear, double zfar,
                   const double world[16], double view_out[16], double proj_out[16]) {
    double aspect = double(width) / double(height);
    dmat4 w = glm::make_mat4(world);
    dmat4 view = glm::inverse(w);
    double pi = glm::pi<double>();
    dmat4 proj = glm::perspective(pi * fovy_deg / 180.0, aspect, znear, zfar);
    std::memcpy(view_out, glm::value_ptr(view), 128);
    std::memcpy(proj_out, glm::value_ptr(proj), 128);
}

// OrbitControls.h:116-135
void glmref_orbit_world(double yaw, double pitch, double radius, const double target[3],
                        double out[16]) {
    dvec3 up = {0, 0, 1};
    dvec3 right = {1, 0, 0};
    dvec3 tgt = {target[0], target[1], target[2]};
    auto translateRadius = glm::translate(dmat4(), dvec3(0.0, 0.0, radius));
    auto translateTarget = glm::translate(dmat4(), tgt);
    auto rotYaw = glm::rotate(yaw, up);
    auto rotPitch = glm::rotate(pitch, right);
    auto flip = dmat4(1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, -1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0);
    dmat4 world = translateTarget * rotYaw * rotPitch * flip * translateRadius;
    std::memcpy(out, glm::value_ptr(world), 128);
}

void glmref_look_at(const double eye[3], const double center[3], const double up[3],
                    double out[16]) {
    dmat4 v = glm::lookAt(dvec3(eye[0], eye[1], eye[2]), dvec3(center[0], center[1], center[2]),
                          dvec3(up[0], up[1], up[2]));
    std::memcpy(out, glm::value_ptr(v), 128);
}

void glmref_inverse(const double m[16], double out[16]) {
    dmat4 r = glm::inverse(glm::make_mat4(m));
    std::memcpy(out, glm::value_ptr(r), 128);
}

// compute_loop_las.h:141-200: UBO (float) and per-file 256 B record
void glmref_file_record(const double view_d[16], const double proj_d[16], const double box_min[3],
                        float transform_out[16], float world_out[16], float view_world_out[16],
                        float proj_out[16]) {
    dmat4 viewd = glm::make_mat4(view_d);
    dmat4 projd = glm::make_mat4(proj_d);
    dmat4 world = glm::translate(dmat4(), dvec3(box_min[0], box_min[1], box_min[2]));
    dmat4 worldViewProj = projd * viewd * world;
    mat4 transform = worldViewProj;
    mat4 fWorld = world;
    mat4 view = viewd;   // uniformData.view = view (float cast of the dmat4)
    mat4 proj = projd;
    mat4 viewWorld = view * fWorld;  // render.cs:204 `uniforms.view * world`
    std::memcpy(transform_out, glm::value_ptr(transform), 64);
    std::memcpy(world_out, glm::value_ptr(fWorld), 64);
    std::memcpy(view_world_out, glm::value_ptr(viewWorld), 64);
    std::memcpy(proj_out, glm::value_ptr(proj), 64);
}

// compute_2021_earlyz.h:108-113 (float products)
void glmref_plain_transform(const double view_d[16], const double proj_d[16], float out[16]) {
    mat4 world;
    mat4 view = glm::make_mat4(view_d);
    mat4 proj = glm::make_mat4(proj_d);
    mat4 worldViewProj = proj * view * world;
    std::memcpy(out, glm::value_ptr(worldViewProj), 64);
}
}
