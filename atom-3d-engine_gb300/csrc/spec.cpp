// spec.cpp — NVRTC build and loading of scene-specialised programs (spec_gen.cpp generates their source).
#include "spec.h"

#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>

#include "tape.h"

// Device sources of the library, embedded at build time (march_kernels.cuh and its includes).
#include "embedded_sources.inc"

namespace mm3e {

namespace {

// ---- NVRTC, loaded on first use -------------------------------------------------------------
struct Nvrtc {
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
    decltype(&nvrtcGetErrorString) error = nullptr;
    std::string status = "not loaded";
};

Nvrtc& nvrtc() {
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
        const char* home = std::getenv("CUDA_HOME");
        for (std::string base : {std::string(home ? home : ""), std::string("/usr/local/cuda")}) {
            if (base.empty()) continue;
            for (const char* dir : {"/lib64/", "/lib/", "/targets/sbsa-linux/lib/", "/targets/x86_64-linux/lib/"}) {
                names.push_back(base + dir + "libnvrtc.so.13");
                names.push_back(base + dir + "libnvrtc.so");
            }
        }
        void* h = nullptr;
        for (const std::string& nm : names)
            if ((h = dlopen(nm.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            n.status = "libnvrtc not found";
            return;
        }
#define MM3E_SYM(field, sym) n.field = reinterpret_cast<decltype(n.field)>(dlsym(h, #sym))
        MM3E_SYM(create, nvrtcCreateProgram);
        MM3E_SYM(compile, nvrtcCompileProgram);
        MM3E_SYM(log_size, nvrtcGetProgramLogSize);
        MM3E_SYM(log, nvrtcGetProgramLog);
        MM3E_SYM(cubin_size, nvrtcGetCUBINSize);
        MM3E_SYM(cubin, nvrtcGetCUBIN);
        MM3E_SYM(destroy, nvrtcDestroyProgram);
        MM3E_SYM(error, nvrtcGetErrorString);
#undef MM3E_SYM
        bool ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy && n.error;
        n.status = ok ? "" : "libnvrtc lacks an entry point";
    });
    return n;
}

std::string embedded(const char* const* chunks) {
    std::string s;
    for (const char* const* c = chunks; *c; ++c) s += *c;
    return s;
}

}  // namespace

std::string nvrtc_status() { return nvrtc().status; }

std::string spec_compile_uncached(const std::string& source, std::vector<char>& cubin);

SpecModule::~SpecModule() {
    if (lib_) cudaLibraryUnload(lib_);
}

// Cubins of programs compiled in this process, by their source text: the same program always
// gives the same cubin, so a scene specialised again (another context or server, a re-lowered
// copy, an autotune candidate seen before) skips NVRTC. Bounded to the most recent 256.
struct CubinCache {
    std::mutex mu;
    std::map<std::string, std::vector<char>> by_source;
    std::deque<std::string> order;
};
CubinCache& cubin_cache() {
    static CubinCache c;
    return c;
}

std::string spec_compile(const std::string& source, std::vector<char>& cubin) {
    Nvrtc& n = nvrtc();
    if (!n.status.empty()) return n.status;
    const char* verbose0 = std::getenv("MM3E_SPEC_VERBOSE");
    const bool cacheable = !(verbose0 && verbose0[0] == '1');
    if (cacheable) {
        CubinCache& cc = cubin_cache();
        std::lock_guard<std::mutex> lk(cc.mu);
        auto it = cc.by_source.find(source);
        if (it != cc.by_source.end()) {
            cubin = it->second;
            return "";
        }
    }
    std::string err = spec_compile_uncached(source, cubin);
    if (cacheable && err.empty() && !cubin.empty()) {
        CubinCache& cc = cubin_cache();
        std::lock_guard<std::mutex> lk(cc.mu);
        if (cc.by_source.emplace(source, cubin).second) {
            cc.order.push_back(source);
            if (cc.order.size() > 256) {
                cc.by_source.erase(cc.order.front());
                cc.order.pop_front();
            }
        }
    }
    return err;
}

std::string spec_compile_uncached(const std::string& source, std::vector<char>& cubin) {
    Nvrtc& n = nvrtc();
    if (!n.status.empty()) return n.status;
    const char* names[] = {"tape.h", "device_math.cuh", "kernels.h", "march_kernels.cuh"};
    std::string bodies[] = {embedded(embed_tape_h), embedded(embed_device_math_cuh), embedded(embed_kernels_h),
                            embedded(embed_march_kernels_cuh)};
    const char* heads[] = {bodies[0].c_str(), bodies[1].c_str(), bodies[2].c_str(), bodies[3].c_str()};
    nvrtcProgram prog = nullptr;
    nvrtcResult r = n.create(&prog, source.c_str(), "mm3e_spec.cu", 4, heads, names);
    if (r != NVRTC_SUCCESS) return std::string("nvrtcCreateProgram: ") + n.error(r);
    // MM3E_SPEC_VERBOSE=1 asks ptxas for its resource report (registers, spills), returned as
    // the log of a successful compile.
    const char* verbose = std::getenv("MM3E_SPEC_VERBOSE");
    bool want_log = verbose && verbose[0] == '1';
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--fmad=false", "-DMM3E_RTC=1",
                          "--ptxas-options=-v"};
    r = n.compile(prog, want_log ? 5 : 4, opts);
    if (r == NVRTC_SUCCESS && want_log) {
        size_t ls = 0;
        n.log_size(prog, &ls);
        std::string log(ls, '\0');
        if (ls) n.log(prog, &log[0]);
        size_t cs = 0;
        n.cubin_size(prog, &cs);
        cubin.assign(cs, 0);
        if (cs) n.cubin(prog, cubin.data());
        n.destroy(&prog);
        return cs ? "LOG:" + log : "NVRTC produced no cubin";
    }
    if (r != NVRTC_SUCCESS) {
        size_t ls = 0;
        n.log_size(prog, &ls);
        std::string log(ls, '\0');
        if (ls) n.log(prog, &log[0]);
        n.destroy(&prog);
        if (log.size() > 4000) log.resize(4000);
        return std::string("NVRTC compile failed: ") + n.error(r) + "\n" + log;
    }
    size_t cs = 0;
    n.cubin_size(prog, &cs);
    cubin.assign(cs, 0);
    if (cs) n.cubin(prog, cubin.data());
    n.destroy(&prog);
    return cs ? "" : "NVRTC produced no cubin";
}

std::string SpecModule::build(const std::string& source, int device, double* compile_ms) {
    auto t0 = std::chrono::steady_clock::now();
    std::vector<char> cubin;
    std::string err = spec_compile(source, cubin);
    if (!err.empty() && err.compare(0, 4, "LOG:") != 0) return err;
    err = load(cubin, device);
    if (!err.empty()) return err;
    if (compile_ms) *compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return "";
}

std::string SpecModule::load(const std::vector<char>& cubin, int device) {
    if (lib_) return "specialised kernels already loaded";
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaLibraryLoadData(&lib_, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    cudaKernel_t km = nullptr, ks = nullptr, ka = nullptr;
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&km, lib_, "mm3e_spec_march");
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&ks, lib_, "mm3e_spec_shadow");
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&ka, lib_, "mm3e_spec_ao");
    if (e != cudaSuccess) return std::string("loading the specialised kernels: ") + cudaGetErrorString(e);
    kernels.march = reinterpret_cast<const void*>(km);
    kernels.shadow = reinterpret_cast<const void*>(ks);
    kernels.ao = reinterpret_cast<const void*>(ka);
    return "";
}

}  // namespace mm3e
