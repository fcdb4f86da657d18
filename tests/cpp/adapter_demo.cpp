// Renders a small scene through include/xgb_xitils.hpp (the C++ adapter with
// Xitils' class names) into a DenoisableRenderTarget and writes the film sums
// to argv[1] as float32 RGB, then the first-hit albedo and normal sums after them.
// The scene matches tests/test_cpp_adapter.py::scene_desc(): a light quad facing
// -y above a Diffuse floor quad and a unit cube (the reference's Cube indices)
// scaled 0.4 and rotated, camera looking along +z.
#include <cmath>
#include <cstdio>
#include <vector>

#include "xgb_xitils.hpp"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const int W = 48, H = 40, SPP = 8;
    try {
        xgb::Context gpu(0);
        // 16-byte stride positions, as xitils::Vector3f arrays are laid out
        float floorPos[4][4] = {{-1, 0, -1, 0}, {1, 0, -1, 0}, {1, 0, 1, 0}, {-1, 0, 1, 0}};
        int quadIdx[6] = {0, 1, 2, 0, 2, 3};
        float lightPos[4][4] = {{-0.25f, 1.5f, -0.25f, 0}, {0.25f, 1.5f, -0.25f, 0}, {0.25f, 1.5f, 0.25f, 0},
                                {-0.25f, 1.5f, 0.25f, 0}};
        float cubePos[8][4];
        for (int i = 0; i < 8; ++i) {
            cubePos[i][0] = i & 1 ? -0.5f : 0.5f;
            cubePos[i][1] = i & 2 ? -0.5f : 0.5f;
            cubePos[i][2] = i & 4 ? -0.5f : 0.5f;
            cubePos[i][3] = 0;
        }
        int cubeIdx[36] = {0, 1, 2, 1, 3, 2, 2, 3, 6, 3, 7, 6, 0, 4, 1, 4, 5, 1,
                           0, 2, 6, 0, 6, 4, 1, 5, 3, 5, 7, 3, 4, 6, 5, 6, 7, 5};
        auto floorMesh = std::make_shared<xgb::TriangleMesh>(gpu);
        floorMesh->setGeometry(4, &floorPos[0][0], nullptr, nullptr, nullptr, nullptr, 6, quadIdx);
        auto lightMesh = std::make_shared<xgb::TriangleMesh>(gpu);
        lightMesh->setGeometry(4, &lightPos[0][0], nullptr, nullptr, nullptr, nullptr, 6, quadIdx);
        auto cubeMesh = std::make_shared<xgb::TriangleMesh>(gpu);
        cubeMesh->setGeometry(8, &cubePos[0][0], nullptr, nullptr, nullptr, nullptr, 36, cubeIdx);
        const float grey[3] = {0.7f, 0.7f, 0.7f}, power[3] = {10.0f, 9.0f, 8.0f}, f0[3] = {0.9f, 0.8f, 0.7f};
        auto diffuse = std::make_shared<xgb::Diffuse>(gpu, grey);
        auto metal = std::make_shared<xgb::Metal>(gpu, 0.3f, f0);
        auto light = std::make_shared<xgb::Emission>(gpu, power);
        xgb::Scene scene(gpu);
        scene.addObject(std::make_shared<xgb::Object>(floorMesh, diffuse, xgb::Transform()));
        scene.addObject(std::make_shared<xgb::Object>(lightMesh, light, xgb::Transform()));
        // transformTRS((0, 0.3, 0), (0, 30, 0), (0.4, 0.4, 0.4)) written out in float: T * R_y(30) * S
        const float c = std::cos(30.0f * 3.14159265f / 180.0f), s = std::sin(30.0f * 3.14159265f / 180.0f);
        float m[16] = {c * 0.4f, 0, s * 0.4f, 0, 0, 0.4f, 0, 0.3f, -s * 0.4f, 0, c * 0.4f, 0, 0, 0, 0, 1};
        float mi[16] = {c / 0.4f, 0, -s / 0.4f, 0, 0, 1 / 0.4f, 0, -0.3f / 0.4f, s / 0.4f, 0, c / 0.4f, 0, 0, 0, 0, 1};
        scene.addObject(std::make_shared<xgb::Object>(cubeMesh, metal, xgb::Transform(m, mi)));
        float cam[16] = {1, 0, 0, 0, 0, 1, 0, 0.6f, 0, 0, 1, -2.5f, 0, 0, 0, 1};
        float camInv[16] = {1, 0, 0, 0, 0, 1, 0, -0.6f, 0, 0, 1, 2.5f, 0, 0, 0, 1};
        scene.setCamera(xgb::PinholeCamera(xgb::Transform(cam, camInv), 0.8f, (float)H / W));
        const float sky[3] = {0.1f, 0.12f, 0.15f};
        scene.setSkyUniform(sky);
        scene.buildAccelerationStructure();
        xgb::DenoisableRenderTarget film(gpu, W, H);
        xgb::StandardPathTracer tracer;
        film.render(scene, SPP / 2, tracer, 0);
        film.render(scene, SPP / 2, tracer, SPP / 2);  // progressive: two sample ranges add up
        std::vector<float> host(4 * W * H);
        film.download(host.data(), 16);  // xitils::Vector3f layout
        FILE* f = std::fopen(argv[1], "wb");
        for (int i = 0; i < W * H; ++i) std::fwrite(&host[4 * i], 4, 3, f);
        film.downloadAlbedo(host.data(), 16);
        for (int i = 0; i < W * H; ++i) std::fwrite(&host[4 * i], 4, 3, f);
        film.downloadNormal(host.data(), 16);
        for (int i = 0; i < W * H; ++i) std::fwrite(&host[4 * i], 4, 3, f);
        std::fclose(f);
        std::printf("ok %d %d %d\n", W, H, SPP);
    } catch (const xgb::Error& e) {
        std::fprintf(stderr, "xgb error %d: %s\n", (int)e.status, e.what());
        return 1;
    }
    return 0;
}
