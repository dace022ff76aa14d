// pt_jit.cu — the megakernel and the wavefront march kernel compiled at run
// time for scenes whose SDF text is not one of the four shipped snippets: the
// reference's InsertSDF +
// GLSLToSPIRV + recompile (src/pathtracer.cpp:2004-2054, 1811-1868, 3836).
// The snippets' translation (pt_glsl.cpp) and a slot dispatcher are compiled
// with NVRTC together with the megakernel's own source, embedded in this
// library at build time (pt_jit_sources.inc), with the flags of the
// precompiled kernels (-fmad=false, IEEE division and square root); the
// cubin is loaded with cudaLibraryLoadData and launched like the precompiled
// megakernel.  Modules are cached per set of snippet texts.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/pt_cuda.h"
#include "pt_jit.h"
#include "pt_jit_sources.inc"  // kJitHeaderNames, kJitHeaderTexts, kJitHeaderCount (generated by build.py)

namespace {

// Fixed-width integer types the headers use (NVRTC defines size_t only);
// LP64 like the host, so shared structs have the host's layout.
const char* kPrelude =
    "typedef unsigned char uint8_t;\n"
    "typedef unsigned short uint16_t;\n"
    "typedef unsigned int uint32_t;\n"
    "typedef int int32_t;\n"
    "typedef unsigned long uint64_t;\n"
    "typedef long int64_t;\n"
    "typedef unsigned long uintptr_t;\n"
    "#define PT_JIT_USER_SDF 1\n";

}  // namespace

namespace {

const char* const kNames[kJitKinds][kJitMaxKernels] = {
    {"ptjit::megakernel<false, 15>", "ptjit::megakernel<true, 15>"},
    {"ptjit::wf_march", nullptr},
    {"ptjit::megakernel<false, 15, double>", "ptjit::megakernel<true, 15, double>"},
};

int kernel_count(JitKind kind) { return kind == kJitMarch ? 1 : 2; }

}  // namespace

std::string pt_jit_program(const std::vector<JitSlot>& slots, JitKind kind) {
    std::string s = kPrelude;
    if (kind == kJitFp64) {
        // The snippets in double: every `float` of the shim and of the
        // translated text is a double (pt_mathf.h is included first so its
        // float functions stay float); the user functions return doubles.
        s += "#include \"../../../include/pt_mathf.h\"\n#define PTG_DOUBLE 1\n#define float double\n";
        s += "#include \"pt_glsl_shim.h\"\n";
        for (const JitSlot& j : slots) s += j.code + "\n";
        s += "#undef float\n";
        s += "template <typename P> static __device__ __forceinline__ double pt_user_sdf_d(int slot, const P& p) {\n"
             "  switch (slot) {\n";
        for (const JitSlot& j : slots)
            s += "    case " + std::to_string(j.slot) + ": return ptg::" + j.prefix + "::" + j.prefix +
                 "sdf(ptg::vec3(p.x, p.y, p.z));\n";
        s += "    default: return 1e5;\n  }\n}\n";
        s += "template <typename P> static __device__ __forceinline__ double pt_user_material_d(int slot, const P& p) {\n"
             "  switch (slot) {\n";
        for (const JitSlot& j : slots)
            s += "    case " + std::to_string(j.slot) + ": return ptg::" + j.prefix + "::" + j.prefix +
                 "sdfmaterial(ptg::vec3(p.x, p.y, p.z));\n";
        s += "    default: return 0.0;\n  }\n}\n";
        s += "#include \"pt_megakernel_body.cuh\"\n";
        return s;
    }
    s += "#include \"pt_glsl_shim.h\"\n";
    for (const JitSlot& j : slots) s += j.code + "\n";
    s += "static __device__ __forceinline__ float pt_user_sdf(int slot, float3 p) {\n  switch (slot) {\n";
    for (const JitSlot& j : slots)
        s += "    case " + std::to_string(j.slot) + ": return ptg::" + j.prefix + "::" + j.prefix +
             "sdf(ptg::vec3(p.x, p.y, p.z));\n";
    s += "    default: return 1e5f;\n  }\n}\n";
    s += "static __device__ __forceinline__ float pt_user_material(int slot, float3 p) {\n  switch (slot) {\n";
    for (const JitSlot& j : slots)
        s += "    case " + std::to_string(j.slot) + ": return ptg::" + j.prefix + "::" + j.prefix +
             "sdfmaterial(ptg::vec3(p.x, p.y, p.z));\n";
    s += "    default: return 0.0f;\n  }\n}\n";
    s += kind == kJitMegakernel ? "#include \"pt_megakernel_body.cuh\"\n" : "#include \"pt_march.cuh\"\n";
    return s;
}

int pt_jit_compile(int device, const std::string& program, JitKind kind, std::vector<char>& cubin,
                   std::string lowered[kJitMaxKernels], std::string& log, bool contract) {
    int major = 0, minor = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device) != cudaSuccess) {
        log = "no CUDA device to compile for";
        return PT_ERR_CUDA;
    }
    return pt_jit_compile_for(major * 10 + minor, program, kind, cubin, lowered, log, contract);
}

int pt_jit_compile_for(int sm, const std::string& program, JitKind kind, std::vector<char>& cubin,
                       std::string lowered[kJitMaxKernels], std::string& log, bool contract) {
    nvrtcProgram prog = nullptr;
    if (nvrtcCreateProgram(&prog, program.c_str(), "pt_jit_kernels.cu", kJitHeaderCount, kJitHeaderTexts,
                           kJitHeaderNames) != NVRTC_SUCCESS) {
        log = "nvrtcCreateProgram failed";
        return PT_ERR_UNSUPPORTED;
    }
    const int nk = kernel_count(kind);
    for (int i = 0; i < nk; i++) nvrtcAddNameExpression(prog, kNames[kind][i]);
    char arch[48];
    std::snprintf(arch, sizeof arch, "--gpu-architecture=sm_%d%s", sm, sm >= 90 ? "a" : "");
    // contract: a*b+c may become one fma (pt_set_fp_contract; not the
    // shader's rounding, so results leave the bit-exact method)
    const char* opts[] = {arch, "--std=c++17", contract ? "--fmad=true" : "--fmad=false", "--prec-div=true",
                          "--prec-sqrt=true", "--ftz=false", "-lineinfo", "-default-device"};
    const nvrtcResult rc = nvrtcCompileProgram(prog, (int)(sizeof opts / sizeof opts[0]), opts);
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    log.assign(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &log[0]);
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return PT_ERR_UNSUPPORTED;
    }
    for (int i = 0; i < nk; i++) {
        const char* low = nullptr;
        if (nvrtcGetLoweredName(prog, kNames[kind][i], &low) != NVRTC_SUCCESS || !low) {
            nvrtcDestroyProgram(&prog);
            log = "kernel name not found in the compiled module";
            return PT_ERR_UNSUPPORTED;
        }
        lowered[i] = low;
    }
    size_t bytes = 0;
    if (nvrtcGetCUBINSize(prog, &bytes) != NVRTC_SUCCESS || bytes == 0) {
        nvrtcDestroyProgram(&prog);
        log = "no cubin";
        return PT_ERR_UNSUPPORTED;
    }
    cubin.resize(bytes);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    return PT_OK;
}

extern "C" int pt_jit_check(const char* const* sources, int n, int sm, char* log, size_t log_cap) {
    if (n < 0 || (n > 0 && !sources) || n > PT_MAX_LIVE_SDFS) return PT_ERR_INVALID;
    std::vector<JitSlot> slots;
    std::string msg;
    int rc = PT_OK;
    for (int i = 0; i < n && rc == PT_OK; i++) {
        JitSlot j;
        rc = pt_jit_translate_slot(sources[i], i, j, msg);
        if (rc == PT_OK) slots.push_back(j);
    }
    std::string all;  // the compiler's messages for both programs
    for (int k = 0; k < kJitKinds && rc == PT_OK; k++) {
        std::vector<char> cubin;
        std::string lowered[kJitMaxKernels];
        // what a context compiles for a scene of these snippets: its march
        // kernel holds no built-in plug-in, and for one snippet the
        // megakernel and march kernel evaluate it without the loop over the
        // SDF set
        const bool fp32 = k == kJitMegakernel || k == kJitMarch;
        const std::string head =
            std::string(fp32 && n == 1 ? "#define PT_ONE_SDF 1\n" : "") +
            (k == kJitMarch ? "#define PT_SDF_KINDS " + std::to_string(1u << PT_SDF_CUSTOM) + "u\n" : "");
        rc = pt_jit_compile_for(sm, head + pt_jit_program(slots, (JitKind)k), (JitKind)k, cubin, lowered, msg);
        all += msg;
    }
    if (log && log_cap) std::snprintf(log, log_cap, "%s", (all.empty() ? msg : all).c_str());
    return rc;
}

int pt_jit_translate_slot(const char* source, int slot, JitSlot& out, std::string& err) {
    out.slot = slot;
    out.prefix = "u" + std::to_string(slot) + "_";
    size_t need = 0;
    char e[256] = {0};
    int rc = pt_glsl_translate(source, out.prefix.c_str(), nullptr, 0, &need, e, sizeof e);
    if (rc != PT_OK) {
        err = e;
        return rc;
    }
    std::string buf(need, '\0');
    rc = pt_glsl_translate(source, out.prefix.c_str(), &buf[0], need, &need, e, sizeof e);
    if (rc != PT_OK) {
        err = e;
        return rc;
    }
    buf.resize(need ? need - 1 : 0);
    out.code = buf;
    return PT_OK;
}

int pt_jit_load(const std::vector<char>& cubin, JitKind kind, const std::string lowered[kJitMaxKernels], JitModule& m,
                std::string& err) {
    cudaError_t e = cudaLibraryLoadData(&m.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    for (int i = 0; i < kernel_count(kind) && e == cudaSuccess; i++)
        e = cudaLibraryGetKernel(&m.kernel[i], m.lib, lowered[i].c_str());
    if (e != cudaSuccess) {
        err = std::string("loading the compiled module: ") + cudaGetErrorString(e);
        if (m.lib) cudaLibraryUnload(m.lib);
        m.lib = nullptr;
        return PT_ERR_CUDA;
    }
    return PT_OK;
}

void pt_jit_unload(JitModule& m) {
    if (m.lib) cudaLibraryUnload(m.lib);
    m.lib = nullptr;
    for (cudaKernel_t& k : m.kernel) k = nullptr;
    m.key.clear();
}

cudaError_t pt_jit_launch(const JitModule& m, const KParams* params, bool trace, cudaStream_t stream) {
    const int W = params->pc.resolution[0], H = params->pc.resolution[1];
    const dim3 block(PT_MK_BLOCK_X, PT_MK_BLOCK_Y);
    const dim3 grid((W + PT_MK_BLOCK_X - 1) / PT_MK_BLOCK_X, (H + PT_MK_BLOCK_Y - 1) / PT_MK_BLOCK_Y);
    void* args[] = {const_cast<KParams*>(params)};
    return cudaLaunchKernel(reinterpret_cast<const void*>(m.kernel[trace ? 1 : 0]), grid, block, args, 0, stream);
}
