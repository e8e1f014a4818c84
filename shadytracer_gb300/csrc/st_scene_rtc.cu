// st_scene_rtc.cu -- a scene given as code, compiled at st_set_scene by NVRTC for sm_103a (the shape-as-code half of
// the reference's scene contract: builder/codegen.js:974-1060 generate -> the scene's SDF and material functions as
// source, compiled by the renderer at setScene, lib/pathtracer/README.md:126-145, core/raytrace_main.js:1145).
//
// THE CONTRACT. The source defines, at file scope, in CUDA C++ over this library's device types (st_device.cuh):
//
//   __device__ float       st_scene_dist(st::f3 p);   the signed distance at p, metres (scene_api.js FOLD_DIST)
//   __device__ st::SceneHit st_scene_full(st::f3 p);  the distance, the material of the nearest surface and the
//                                                     medium (the least-deep item p is inside; 0 the air) (FOLD_FULL)
//
// and, optionally, with `#define ST_SCENE_COUNTS`, a twin of the distance that tallies its work for the counting pass:
//
//   __device__ float st_scene_dist_count(st::f3 p, uint32_t* wc);    (st_device.cuh WC_*: wc_prim / wc_test)
//
// The library compiles it together with the kernels that ask the scene (st_scene_kernels.cuh: the march, the
// surface, the occlusion pass, the emitter rays' resolve, the step cache's fill, the distance at points) under the
// CodeScene policy below -- the scene's functions inlined into each kernel, no table in shared memory -- and loads
// the result as a library. The build flags are the library's own (fast f32 division and square root, denormals
// flushed). An error is reported with the line of the scene's source it names and that line's text (the emitter
// tags each primitive's code with its item and node), and the previous scene is kept.
//
// COMPILED ONCE. A source compiled before in this process (the same text) is loaded from a cache of its cubin.
#include <dlfcn.h>
#include <nvrtc.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "st_internal.h"

namespace st {
namespace {

// the module's text around the scene's source: the integer types NVRTC lacks, the kernels' header, the scene, then
// the policy and the kernels named for instantiation
const char* kPrelude =
    "typedef unsigned char uint8_t; typedef unsigned short uint16_t; typedef unsigned int uint32_t;\n"
    "typedef unsigned long long uint64_t; typedef signed char int8_t; typedef short int16_t; typedef int int32_t;\n"
    "typedef long long int64_t;\n"
    "#include \"st_scene_kernels.cuh\"\n"
    "#line 1 \"scene\"\n";
const char* kPolicy =
    "\n#line 1 \"st_scene_code\"\n"
    "namespace st {\n"
    "struct CodeScene {\n"
    "    static constexpr bool kTable = false;\n"
    "    template <bool COUNT>\n"
    "    __device__ static __forceinline__ float dist(const DPrim*, uint32_t, f3 p, uint32_t* wc) {\n"
    "#ifdef ST_SCENE_COUNTS\n"
    "        if (COUNT) return ::st_scene_dist_count(p, wc);\n"
    "#endif\n"
    "        return ::st_scene_dist(p);\n"
    "    }\n"
    "    __device__ static __forceinline__ float dist(const DPrim*, uint32_t, f3 p) { return ::st_scene_dist(p); }\n"
    "    __device__ static __forceinline__ SceneHit full(const DPrim*, uint32_t, f3 p) { return ::st_scene_full(p); }\n"
    "};\n"
    "}  // namespace st\n";

// the kernels the library launches for a code scene, by the name expressions NVRTC instantiates
const char* kNames[] = {
    "st::k_march<st::CodeScene, false, false, false>", "st::k_march<st::CodeScene, false, false, true>",
    "st::k_march<st::CodeScene, true, false, false>",  "st::k_march<st::CodeScene, true, false, true>",
    "st::k_surface<st::CodeScene>",  "st::k_occlude<st::CodeScene, 0>", "st::k_occlude<st::CodeScene, 1>",
    "st::k_emit_resolve<st::CodeScene>", "st::k_sc_fill<st::CodeScene>", "st::k_eval_sdf<st::CodeScene>",
};
constexpr int kNumNames = (int)(sizeof(kNames) / sizeof(kNames[0]));

struct Compiled {
    std::vector<char> cubin;
    std::vector<std::string> lowered;
    double ms = 0.0;
};
std::mutex g_cache_mutex;
std::unordered_map<std::string, Compiled> g_cache;     // by the module's full text

// where this library's sources lie: csrc beside the .so (shadytracer_gb300/libshadytracer.so, .../csrc)
std::string csrc_dir() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&csrc_dir), &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        const size_t cut = so.find_last_of('/');
        return (cut == std::string::npos ? std::string(".") : so.substr(0, cut)) + "/csrc";
    }
    return "csrc";
}

// NVRTC's log with each error on the scene's source followed by that line's text
std::string map_log(const std::string& log, const std::string& src) {
    std::vector<std::string> lines;
    {
        std::stringstream ss(src);
        std::string l;
        while (std::getline(ss, l)) lines.push_back(l);
    }
    std::stringstream in(log), out;
    std::string l;
    while (std::getline(in, l)) {
        if (l.empty()) continue;
        out << l << "\n";
        if (l.compare(0, 6, "scene(") == 0) {
            const int n = std::atoi(l.c_str() + 6);
            if (n >= 1 && n <= (int)lines.size()) out << "    at scene line " << n << ": " << lines[n - 1] << "\n";
        }
    }
    return out.str();
}

bool compile(const std::string& module, const std::string& user, Compiled& c, std::string& err) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, module.c_str(), "st_scene_module.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        err = "NVRTC could not create the program";
        return false;
    }
    for (int i = 0; i < kNumNames; i++) nvrtcAddNameExpression(prog, kNames[i]);
    const std::string inc = "--include-path=" + csrc_dir();
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device", "--prec-div=false",
                          "--prec-sqrt=false", "--ftz=true", "-lineinfo", inc.c_str()};
    const auto t0 = std::chrono::steady_clock::now();
    const nvrtcResult r = nvrtcCompileProgram(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
    c.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    std::string log(ls, '\0');
    if (ls) nvrtcGetProgramLog(prog, &log[0]);
    while (!log.empty() && log.back() == '\0') log.pop_back();
    if (r != NVRTC_SUCCESS) {
        err = std::string("the scene's code did not compile (") + nvrtcGetErrorString(r) + "):\n" + map_log(log, user);
        nvrtcDestroyProgram(&prog);
        return false;
    }
    size_t cs = 0;
    nvrtcGetCUBINSize(prog, &cs);
    c.cubin.resize(cs);
    if (!cs || nvrtcGetCUBIN(prog, c.cubin.data()) != NVRTC_SUCCESS) {
        err = "NVRTC gave no cubin for sm_103a";
        nvrtcDestroyProgram(&prog);
        return false;
    }
    c.lowered.clear();
    for (int i = 0; i < kNumNames; i++) {
        const char* low = nullptr;
        if (nvrtcGetLoweredName(prog, kNames[i], &low) != NVRTC_SUCCESS || !low) {
            err = std::string("NVRTC did not instantiate ") + kNames[i];
            nvrtcDestroyProgram(&prog);
            return false;
        }
        c.lowered.push_back(low);
    }
    nvrtcDestroyProgram(&prog);
    return true;
}

}  // namespace

// the scene's module compiled, or found in the cache; cached says which
static bool compiled_for(const char* user_src, Compiled& c, bool& cached, std::string& err) {
    const std::string user = user_src ? user_src : "";
    if (user.find("st_scene_dist") == std::string::npos || user.find("st_scene_full") == std::string::npos) {
        err = "a scene's code defines st_scene_dist and st_scene_full";
        return false;
    }
    const std::string module = std::string(kPrelude) + user + kPolicy;
    cached = false;
    {
        std::lock_guard<std::mutex> lock(g_cache_mutex);
        auto it = g_cache.find(module);
        if (it != g_cache.end()) { c = it->second; cached = true; }
    }
    if (!cached) {
        if (!compile(module, user, c, err)) return false;
        std::lock_guard<std::mutex> lock(g_cache_mutex);
        g_cache[module] = c;
    }
    return true;
}

bool scene_code_compile(const char* user_src, double& ms, std::string& err) {
    Compiled c;
    bool cached = false;
    if (!compiled_for(user_src, c, cached, err)) return false;
    ms = cached ? 0.0 : c.ms;
    return true;
}

// the scene's source compiled (or found in the cache) and loaded; on failure err says why and nothing is kept
bool scene_code_build(const char* user_src, SceneCode& out, std::string& err) {
    Compiled c;
    bool cached = false;
    if (!compiled_for(user_src, c, cached, err)) return false;
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, c.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        err = std::string("loading the scene's compiled code: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return false;
    }
    const void* k[kNumNames] = {};
    for (int i = 0; i < kNumNames; i++) {
        cudaKernel_t kk = nullptr;
        e = cudaLibraryGetKernel(&kk, lib, c.lowered[i].c_str());
        if (e != cudaSuccess) {
            err = std::string("the scene's kernel ") + kNames[i] + ": " + cudaGetErrorString(e);
            cudaGetLastError();
            cudaLibraryUnload(lib);
            return false;
        }
        k[i] = reinterpret_cast<const void*>(kk);
    }
    out = SceneCode{};
    out.lib = lib;
    out.march[0][0] = k[0]; out.march[0][1] = k[1]; out.march[1][0] = k[2]; out.march[1][1] = k[3];
    out.surface = k[4];
    out.occlude[0] = k[5]; out.occlude[1] = k[6];
    out.emit_resolve = k[7];
    out.sc_fill = k[8];
    out.eval_sdf = k[9];
    out.compile_ms = cached ? 0.0 : c.ms;
    out.cubin_bytes = c.cubin.size();
    return true;
}

void scene_code_free(SceneCode& c) {
    if (c.lib) cudaLibraryUnload(reinterpret_cast<cudaLibrary_t>(c.lib));
    c = SceneCode{};
}

}  // namespace st

// a scene's code compiled into the process's cache, no device needed (include/shadytracer.h st_compile_scene)
extern "C" int st_compile_scene(const char* cuda_src, char* errbuf, size_t errlen, double* compile_ms) {
    if (!cuda_src) return ST_ERR_ARG;
    double ms = 0.0;
    std::string err;
    const bool ok = st::scene_code_compile(cuda_src, ms, err);
    if (compile_ms) *compile_ms = ms;
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", ok ? "" : err.c_str());
    return ok ? ST_OK : ST_ERR_COMPILE;
}
