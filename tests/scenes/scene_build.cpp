// Scene library (libjsbscene.so): seeded synthetic workloads serialised as "JSBS" scenes, with every
// body's settings bytes written by the SoftBodySharedSettings mirror (shared_settings.cpp).
// TEST AND BENCHMARK INFRASTRUCTURE: the tests, the benchmark and the smoke check load it to make
// their inputs; the product library (libjsb.so) neither links nor calls it. Its output is byte for
// byte what Jolt's own CreateConstraints / Optimize / SaveBinaryState write for the same scene
// (tests/test_settings_mirror.py, and a SHA-256 of every full-size scene in the golden fixtures).

#include <cstring>
#include <exception>
#include <string>

#include "scene_io.h"
#include "shared_settings.h"

namespace {
thread_local std::string g_error;
}

extern "C" {

// Last error message of the calling thread.
const char *scene_last_error(void) { return g_error.c_str(); }

// Serialises scene `name` ("pinned_cloth" | "uneven_batch" | "large_cloth" | "diff_cloth" |
// "diff_batch") with the space-separated "key=value" parameters `params`. Call with out == NULL to
// query *len. Returns 0 on success, 1 on an unknown scene or bad argument, 2 when the buffer is too small.
int scene_build(const char *name, const char *params, void *out, size_t capacity, size_t *len) {
    using namespace jsb;
    if (!name || !len) {
        g_error = "null argument";
        return 1;
    }
    scene::SceneSpec spec;
    try {
        if (!scene::make_named_scene(name, params ? params : "", spec)) {
            g_error = std::string("unknown scene ") + name;
            return 1;
        }
        std::string bytes =
            scene::serialize_scene(spec, [](const scene::MeshSpec &m) { return host::build_settings(m).SaveBinaryState(); });
        *len = bytes.size();
        if (!out) return 0;
        if (capacity < bytes.size()) {
            g_error = "output buffer too small";
            return 2;
        }
        memcpy(out, bytes.data(), bytes.size());
    } catch (const std::exception &e) {
        g_error = std::string("scene build failed: ") + e.what();
        return 1;
    }
    return 0;
}

}  // extern "C"
