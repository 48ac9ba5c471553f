// RayTracer.h — the drop-in RayTracer (the reference's RayTracer.h:16-57): same mode macros,
// same public members and the same asynchronous start() / stop() / isFinish / useTime
// contract, rendering on the GPU through the C ABI (include/rt_gb300.h) instead of CPU
// threads. `output` keeps the reference layout: 2048*2048*3 bytes, rows bottom-up with a
// stride of 3*width, only the 64x64 tiles inside width x height written (RayTracer.cpp:13-37).
#pragma once
#include <atomic>
#include <string>
#include <thread>

#include "../../include/rt_gb300.h"
#include "Flatten.h"
#include "Scene.h"

#define MY_MODEL_CHECK 0x1
#define MY_MODEL_DEPTHTEST 0x2
#define MY_MODEL_NORMALTEST 0x3
#define MY_MODEL_TEXTURETEST 0x4
#define MY_MODEL_MATERIALTEST 0x5
#define MY_MODEL_SHADOWTEST 0x6
#define MY_MODEL_REFLECTTEST 0x7
#define MY_MODEL_REFRACTTEST 0x8
#define MY_MODEL_RAYTRACE 0x80

class RayTracer
{
private:
    Scene *scene;
    rt_ctx *ctx = nullptr;
    std::thread worker;
    FlatScene flat;
    std::atomic<int> status_{RT_OK};
    std::string error_;
    int device_ = 0;
public:
    unsigned int texID = 0;
    uint8_t *output;
    // the reference declares `volatile bool`; an atomic keeps every use of it (`if
    // (!rt.isFinish)`, polling loops, assignment) and orders the render thread's writes of
    // `output`, `useTime` and the status before the flag, which volatile does not on Arm
    std::atomic<bool> isFinish{true};
    volatile double useTime = 0.0;
    uint8_t maxLevel = 1;
    int width = 0, height = 0;

    RayTracer(Scene &scene, int device = 0);
    ~RayTracer();
    RayTracer(const RayTracer &) = delete;
    RayTracer &operator=(const RayTracer &) = delete;

    // render the scene's camera view in the given mode; tnum (CPU threads in the reference) is
    // accepted and ignored. Returns at once; isFinish turns true when output is complete.
    void start(const uint8_t type, const int8_t tnum = 1);
    // cooperative cancel of a running render (RayTracer.cpp:698-701)
    void stop();
    // RT_OK or the RT_ERR_* code of the last render, and its message
    int status() const { return status_.load(); }
    const std::string &lastError() const { return error_; }
};
