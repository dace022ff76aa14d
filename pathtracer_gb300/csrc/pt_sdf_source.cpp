// pt_sdf_source.cpp — decoding of SDF plug-in sources for pt_set_sdfs.
//
// The reference compiles each scene's `sdf[i].glsl` into the shader at run
// time (InsertSDF + GLSLToSPIRV, src/pathtracer.cpp:2004-2054, 1811-1868).
// Here the four shipped snippets are CUDA __device__ functions, and a source
// string selects one of them in one of two forms:
//   * the snippet's GLSL text: recognised by the FNV-1a-64 hash of the text
//     with every whitespace run collapsed to one space (so CRLF/LF and
//     indentation do not matter).  The table holds the hashes of the four
//     files in sdfs/ and of the copies carried by scenes/scene3..7.json, whose
//     sdfmaterial() differ only in material constants; it was generated by
//     tests/golden/gen_sdf_fingerprints.py.
//   * "builtin:<name>[:m0[,m1[,m2]]]" with name in blob, mandelbulb,
//     mandelbulb_const, menger, terrain and optional material constants.
#include <cctype>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/pt_cuda.h"

namespace {

struct Fingerprint {
    uint64_t hash;
    pt_sdf_plugin plugin;
};

// {hash, {kind, material_mode, {material}}}
const Fingerprint kFingerprints[] = {
    {0x6de57505fc723c7eull, {PT_SDF_BLOB, PT_SDFMAT_DEFAULT, {4.0f, 5.0f, 6.0f}}},        // sdfs/blob.glsl
    {0xdcc8f6bccda6d8d9ull, {PT_SDF_MANDELBULB, PT_SDFMAT_DEFAULT, {4.0f, 3.0f, 0.0f}}},  // sdfs/mandelbulb.glsl
    {0x3c94eee4f8b59872ull, {PT_SDF_MENGER, PT_SDFMAT_CONSTANT, {0.0f, 0.0f, 0.0f}}},     // sdfs/menger.glsl
    {0x742b6d88271746b9ull, {PT_SDF_TERRAIN, PT_SDFMAT_CONSTANT, {0.0f, 0.0f, 0.0f}}},    // sdfs/terrain.glsl
    {0xe86f17a11e62fd66ull, {PT_SDF_BLOB, PT_SDFMAT_DEFAULT, {3.0f, 4.0f, 5.0f}}},        // scenes/scene3.json, scene5.json
    {0x5e591c833348e2e0ull, {PT_SDF_MANDELBULB, PT_SDFMAT_CONSTANT, {3.0f, 0.0f, 0.0f}}}, // scenes/scene4.json
    {0x02cb7b03b6d3b701ull, {PT_SDF_MANDELBULB, PT_SDFMAT_DEFAULT, {3.0f, 2.0f, 0.0f}}},  // scenes/scene6.json
    {0xc8ce1f6bb7bbc161ull, {PT_SDF_MANDELBULB, PT_SDFMAT_DEFAULT, {5.0f, 4.0f, 0.0f}}},  // scenes/scene7.json
};

uint64_t normalized_fnv1a(const char* s) {
    uint64_t h = 0xcbf29ce484222325ull;
    auto feed = [&h](unsigned char c) {
        h ^= c;
        h *= 0x100000001b3ull;
    };
    bool pending_space = false, any = false;
    for (const unsigned char* p = (const unsigned char*)s; *p; ++p) {
        if (std::isspace(*p)) {
            pending_space = any;
            continue;
        }
        if (pending_space) feed(' ');
        pending_space = false;
        any = true;
        feed(*p);
    }
    return h;
}

bool parse_builtin(const char* s, pt_sdf_plugin* out) {
    const char* prefix = "builtin:";
    if (std::strncmp(s, prefix, std::strlen(prefix)) != 0) return false;
    std::string rest(s + std::strlen(prefix));
    std::string name = rest, params;
    const size_t colon = rest.find(':');
    if (colon != std::string::npos) {
        name = rest.substr(0, colon);
        params = rest.substr(colon + 1);
    }
    pt_sdf_plugin p{};
    if (name == "blob") {
        p = {PT_SDF_BLOB, PT_SDFMAT_DEFAULT, {4.0f, 5.0f, 6.0f}};
    } else if (name == "mandelbulb") {
        p = {PT_SDF_MANDELBULB, PT_SDFMAT_DEFAULT, {4.0f, 3.0f, 0.0f}};
    } else if (name == "mandelbulb_const") {
        p = {PT_SDF_MANDELBULB, PT_SDFMAT_CONSTANT, {3.0f, 0.0f, 0.0f}};
    } else if (name == "menger") {
        p = {PT_SDF_MENGER, PT_SDFMAT_CONSTANT, {0.0f, 0.0f, 0.0f}};
    } else if (name == "terrain") {
        p = {PT_SDF_TERRAIN, PT_SDFMAT_CONSTANT, {0.0f, 0.0f, 0.0f}};
    } else {
        return false;
    }
    int idx = 0;
    const char* c = params.c_str();
    while (*c && idx < 3) {
        char* end = nullptr;
        const float v = std::strtof(c, &end);
        if (end == c) return false;
        p.material[idx++] = v;
        c = end;
        if (*c == ',') ++c;
        else if (*c) return false;
    }
    *out = p;
    return true;
}

}  // namespace

extern "C" int pt_parse_sdf_source(const char* source, pt_sdf_plugin* out) {
    if (!source || !out) return PT_ERR_INVALID;
    if (parse_builtin(source, out)) return PT_OK;
    const uint64_t h = normalized_fnv1a(source);
    for (const Fingerprint& f : kFingerprints) {
        if (f.hash == h) {
            *out = f.plugin;
            return PT_OK;
        }
    }
    return PT_ERR_UNSUPPORTED;
}

extern "C" uint64_t pt_sdf_source_fingerprint(const char* source) { return source ? normalized_fnv1a(source) : 0; }
