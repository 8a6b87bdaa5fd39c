// A reference-style frame loop over include/cr_method.hpp, used by the tests.
//
//   method_demo info
//       prints "name|group|description" of every registered method (host only)
//   method_demo render <view+proj.f64> <out.u32> <method> <n> <seed> <extent> <W> <H>
//       generates the seeded terrain on the GPU, registers the three batched
//       methods, selects <method> by name, runs update() + render() twice (the
//       second frame must equal the first: the fb is re-cleared after resolve)
//       and writes the RGBA8 image
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "cr_method.hpp"
#include "cr_synth.h"

static int fail(const char* what, cr_status s) {
    std::fprintf(stderr, "%s: %s\n", what, cr_status_string(s));
    return 1;
}

int main(int argc, char** argv) {
    const char* names[] = {"loop_las",       "loop_las_prefetch", "loop_las_hqs",
                           "(2021) early-z", "(2021) dedup",      "(2021) early-z & reduce"};
    if (argc == 2 && std::strcmp(argv[1], "info") == 0) {
        for (const char* n : names) {
            std::string name, group, desc;
            if (!cr::method_info(n, nullptr, &name, &group, &desc)) return 2;
            std::printf("%s|%s|%s\n", name.c_str(), group.c_str(), desc.c_str());
        }
        return cr::method_info("no such method", nullptr, nullptr, nullptr, nullptr) ? 3 : 0;
    }
    if (argc != 10 || std::strcmp(argv[1], "render") != 0) return 4;
    cr::ViewTarget t;
    FILE* f = std::fopen(argv[2], "rb");
    if (!f || std::fread(t.view, 8, 16, f) != 16 || std::fread(t.proj, 8, 16, f) != 16) return 5;
    std::fclose(f);
    const long long n = std::atoll(argv[5]);
    t.width = std::atoi(argv[8]);
    t.height = std::atoi(argv[9]);

    cr_ctx* ctx = nullptr;
    cr_status s = cr_ctx_create(0, &ctx);
    if (s != CR_OK) return fail("ctx", s);
    cr_cloud* cloud = nullptr;
    s = cr_cloud_create(ctx, n, cr_num_batches(n), 1, CR_STREAM_ALL, &cloud);
    if (s != CR_OK) return fail("cloud", s);
    cr_synth_params sp;
    cr_synth_params_default(CR_SYNTH_TERRAIN, std::atof(argv[7]), std::strtoull(argv[6], nullptr, 10), &sp);
    cr_las_header hdr;
    s = cr_synth_cloud_device(ctx, &sp, n, cloud, &hdr, nullptr);
    if (s != CR_OK) return fail("synth", s);

    cr::MethodRegistry runtime;
    for (int i = 0; i < 3; i++) {
        auto m = std::make_unique<cr::RasterMethod>(ctx, names[i]);
        m->set_cloud(cloud);
        runtime.add(std::move(m));
    }
    cr::Method* m = runtime.select(argv[4]);
    if (!m) return 6;
    std::vector<uint32_t> first((size_t)t.width * t.height), img((size_t)t.width * t.height);
    for (int frame = 0; frame < 2; frame++) {
        m->update();
        m->render(t, nullptr);
        auto* rm = static_cast<cr::RasterMethod*>(m);
        if (rm->last_status() != CR_OK) return fail(rm->last_error().c_str(), rm->last_status());
        s = rm->read_image(frame == 0 ? first.data() : img.data(), nullptr);
        if (s != CR_OK) return fail("read", s);
        s = cr_ctx_check(ctx, nullptr);
        if (s != CR_OK) return fail("check", s);
    }
    if (first != img) return 7;
    f = std::fopen(argv[3], "wb");
    if (!f || std::fwrite(img.data(), 4, img.size(), f) != img.size()) return 8;
    std::fclose(f);
    runtime = cr::MethodRegistry();
    cr_cloud_destroy(ctx, cloud);
    cr_ctx_destroy(ctx);
    return 0;
}
