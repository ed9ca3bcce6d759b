// File readers of the host-compiled device-code checks (tests/host_checks.py): the
// lowered tape and payloads as 16-byte words, float arrays (points, rays) and a camera, each read
// whole from the files the test writes. Test infrastructure only.
#pragma once
#include <cstdio>
#include <vector>

#include "kernels.h"

// The whole file as 16-byte words, 16-byte aligned as on the device, with zero words after it.
inline std::vector<float4> read_words(const char* path) {
    std::vector<float4> w;
    FILE* f = std::fopen(path, "rb");
    if (!f) return w;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    w.assign((size_t)n / sizeof(float4) + 64, make_float4(0.f, 0.f, 0.f, 0.f));
    const size_t got = std::fread(w.data(), 1, (size_t)n, f);
    (void)got;
    std::fclose(f);
    return w;
}

inline std::vector<float> read_floats(const char* path) {
    std::vector<float> v;
    FILE* f = std::fopen(path, "rb");
    if (!f) return v;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    v.resize((size_t)n / sizeof(float));
    const size_t got = std::fread(v.data(), sizeof(float), v.size(), f);
    (void)got;
    std::fclose(f);
    return v;
}

// Camera as 13 floats: eye, forward, right, up, fov_scale.
inline mm3e::CameraArgs read_camera(const char* path) {
    const std::vector<float> c = read_floats(path);
    mm3e::CameraArgs cam{};
    for (int k = 0; k < 3 && c.size() >= 13; ++k) {
        cam.eye[k] = c[k];
        cam.fwd[k] = c[3 + k];
        cam.right[k] = c[6 + k];
        cam.up[k] = c[9 + k];
    }
    if (c.size() >= 13) cam.fov_scale = c[12];
    return cam;
}
