// Headless stand-in for the reference's Win32/Direct3D-11 platform header.
//
// Test infrastructure only: the reference renderer (`Renderer.h`) includes
// "ThirdParty/GamesEngineering/GamesEngineeringBase.h" for a window it draws
// tonemapped pixels into (`Renderer.h:706`), a timer (`main.cpp:414`) and
// `GetSystemInfo` for its thread count (`Renderer.h:256-258`).  This file
// provides the same names with a plain byte buffer as the "window", so the
// reference's CPU path compiles and runs on Linux for the oracle.
// It is found before the reference's own header because the oracle build
// passes this directory ahead of the reference sources with `-I-`.
#pragma once

#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#ifndef VK_ESCAPE
#define VK_ESCAPE 0x1B
#endif

// Thread count the reference's RayTracer::init reads; the harness sets it.
inline unsigned int& pgx_ref_thread_count() {
    static unsigned int n = 0;
    return n;
}

struct SYSTEM_INFO {
    unsigned int dwNumberOfProcessors;
};

inline void GetSystemInfo(SYSTEM_INFO* info) {
    unsigned int n = pgx_ref_thread_count();
    if (n == 0) n = std::thread::hardware_concurrency();
    if (n == 0) n = 1;
    info->dwNumberOfProcessors = n;
}

namespace GamesEngineeringBase {

class Window {
  public:
    void create(unsigned int w, unsigned int h, const std::string&, bool = false, int = 0, int = 0) {
        width = w;
        height = h;
        pixels.assign(static_cast<size_t>(w) * h * 3, 0);
    }
    void draw(int x, int y, unsigned char r, unsigned char g, unsigned char b) {
        if (x < 0 || y < 0 || x >= static_cast<int>(width) || y >= static_cast<int>(height)) return;
        size_t i = (static_cast<size_t>(y) * width + x) * 3;
        pixels[i] = r;
        pixels[i + 1] = g;
        pixels[i + 2] = b;
    }
    unsigned int getWidth() const { return width; }
    unsigned int getHeight() const { return height; }
    unsigned char* getBackBuffer() { return pixels.data(); }
    void checkInput() {}
    void clear() { std::fill(pixels.begin(), pixels.end(), 0); }
    void present() {}
    bool keyPressed(int) const { return false; }

  private:
    unsigned int width = 0, height = 0;
    std::vector<unsigned char> pixels;
};

class Timer {
  public:
    Timer() { reset(); }
    void reset() { start = std::chrono::steady_clock::now(); }
    float dt() {
        auto now = std::chrono::steady_clock::now();
        float s = std::chrono::duration<float>(now - start).count();
        start = now;
        return s;
    }

  private:
    std::chrono::steady_clock::time_point start;
};

}  // namespace GamesEngineeringBase
