// Stand-in for stb_image.h (the reference's ThirdParty/stb is empty in this
// checkout). TEST INFRASTRUCTURE ONLY.
//
// The CPU checker never decodes image files. Instead the harness registers
// float RGB arrays under names like "mem:3"; stbi_loadf hands back a malloc'd
// copy, so xitils::Texture(const std::string&) and SkySphereFromImage run their
// own constructors unchanged. Any other name fails loudly.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#define STBI_rgb 3

struct stbi_mem_image {
    int width = 0, height = 0;
    std::vector<float> rgb;  // width * height * 3
};

inline std::map<std::string, stbi_mem_image>& stbi_mem_registry() {
    static std::map<std::string, stbi_mem_image> registry;
    return registry;
}

inline float* stbi_loadf(const char* filename, int* w, int* h, int* comp, int req_comp) {
    auto& reg = stbi_mem_registry();
    auto it = reg.find(filename);
    if (it == reg.end() || req_comp != STBI_rgb) {
        std::fprintf(stderr, "oracle shim: no in-memory image named %s\n", filename);
        std::abort();
    }
    const stbi_mem_image& img = it->second;
    *w = img.width;
    *h = img.height;
    *comp = 3;
    float* out = (float*)std::malloc(img.rgb.size() * sizeof(float));
    std::memcpy(out, img.rgb.data(), img.rgb.size() * sizeof(float));
    return out;
}
inline void stbi_image_free(void* p) { std::free(p); }
