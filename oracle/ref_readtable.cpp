// ORACLE — test infrastructure only.
//
// Harness around the reference's own sounding reader: Game/readTable.cpp (readKNMIFile :27-132,
// readDWDFile :134-354, initEnvironment :364-474) and Engine/source/math/meteoformulas.cpp,
// compiled unmodified from the reference checkout. This file is appended to a generated
// translation unit that first fixes the compile-time grid (Game/config.h) and includes
// Game/readTable.cpp; it supplies what the reader needs from the rest of the game:
//   * the `Game` object, whose environmentGPU::init (Game/environment.cuh:42) is replaced by a
//     capture of its seven arrays;
//   * bee::Engine.DebugRenderer() for the skew-T plot (never called here).
// The C functions below are called through ctypes by the golden-vector generator.
#include <cstring>
#include <stdexcept>

namespace bee {
EngineStub Engine;
bee::DebugRenderer& EngineStub::DebugRenderer() { throw std::runtime_error("no debug renderer"); }
void DebugRenderer::AddLine(DebugCategory::Enum, const glm::vec3&, const glm::vec3&, const glm::vec4&) {}
void DebugRenderer::AddCircle(DebugCategory::Enum, const glm::vec3&, float, const glm::vec3&, const glm::vec4&) {}
}  // namespace bee

namespace {
struct Capture {
    float* theta = nullptr;
    float* vel = nullptr;
    float* qv = nullptr;
    float* ground_T = nullptr;
    float* ground_p = nullptr;
    float* p3d = nullptr;
    float* p_column = nullptr;
    int calls = 0;
} g_cap;
environmentGPU* g_env = nullptr;
readTable* g_table = nullptr;
}  // namespace

environmentGPU::environmentGPU() {}
environmentGPU::~environmentGPU() {}
void environmentGPU::init(float* potTemps, glm::vec3* velField, float* Qv, float* groundTemp, float* groundPres,
                          float* pressures, float* smallPressure) {
    std::memcpy(g_cap.theta, potTemps, sizeof(float) * GRIDSIZESKY);
    std::memcpy(g_cap.vel, velField, sizeof(float) * 3 * GRIDSIZESKY);
    std::memcpy(g_cap.qv, Qv, sizeof(float) * GRIDSIZESKY);
    std::memcpy(g_cap.ground_T, groundTemp, sizeof(float) * GRIDSIZEGROUND);
    std::memcpy(g_cap.ground_p, groundPres, sizeof(float) * GRIDSIZEGROUND);
    std::memcpy(g_cap.p3d, pressures, sizeof(float) * GRIDSIZESKY);
    std::memcpy(g_cap.p_column, smallPressure, sizeof(float) * GRIDSIZESKYY);
    g_cap.calls++;
}

game::game() { m_envGPUObj = g_env = new environmentGPU(); }
game::~game() {}
game Game;

extern "C" {

int ref_grid(int* X, int* Y, int* Z, float* voxel) {
    *X = GRIDSIZESKYX;
    *Y = GRIDSIZESKYY;
    *Z = GRIDSIZESKYZ;
    *voxel = VOXELSIZE;
    return 0;
}

// 0 = KNMI (readKNMIFile), 1 = DWD (readDWDFile). Returns the number of sounding rows read.
long ref_read(int kind, const char* path) {
    delete g_table;
    g_table = new readTable();
    if (kind == 0) g_table->readKNMIFile(path);
    else g_table->readDWDFile(path);
    return (long)g_table->skewTData.data.dataSize;
}

// The six sounding columns of the last ref_read, each n values.
int ref_rows(float* altitude, float* pressure, float* temperature, float* dew_point, float* wind_speed, float* wind_dir) {
    const radioSondeData& d = g_table->skewTData.data;
    const size_t n = d.dataSize;
    std::memcpy(altitude, d.altitude, n * sizeof(float));
    std::memcpy(pressure, d.pressure, n * sizeof(float));
    std::memcpy(temperature, d.temperature, n * sizeof(float));
    std::memcpy(dew_point, d.dewPoint, n * sizeof(float));
    std::memcpy(wind_speed, d.windSpeed, n * sizeof(float));
    std::memcpy(wind_dir, d.windDir, n * sizeof(float));
    return 0;
}

// readTable::initEnvironment on the last ref_read; the outputs are what it hands to init.
int ref_init_environment(float* theta, float* vel, float* qv, float* ground_T, float* ground_p, float* p3d,
                         float* p_column) {
    g_cap.theta = theta;
    g_cap.vel = vel;
    g_cap.qv = qv;
    g_cap.ground_T = ground_T;
    g_cap.ground_p = ground_p;
    g_cap.p3d = p3d;
    g_cap.p_column = p_column;
    const int before = g_cap.calls;
    g_table->initEnvironment();
    return g_cap.calls - before;
}

}  // extern "C"
