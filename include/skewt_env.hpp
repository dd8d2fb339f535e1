// skewt_env.hpp — C++ adapter with the shape of the reference's environmentGPU class
// (Game/environment.cuh:9-183), over the C ABI in skewt.h. Header-only; link libskewt_gb300.so.
//
// The reference's call sites map one to one:
//   Game.EnvGPU().init(potTemp, velField, Qv, groundTemp, groundPressure, pressures, pressuresSmall)
//       (Game/readTable.cpp:470)                        -> env.init(...)
//   Game.EnvGPU().updateGPU(dt, speed)  (Game/game.cpp:56) -> env.updateGPU(dt, speed)
//   getParamArray(parameter, direction) (Game/environment.cu:1076) -> env.getParamArray(...)
//   editor::GPUSetEnv per-step readback (Game/editor.cpp:226)       -> env.readField(...)
//   Game.ReadTable().readDWDFile(file) / readKNMIFile(file) / initEnvironment()
//       (Game/gameSystem.cpp:43-47)  -> table.readDWDFile(file, reader, ctx) / ... / table.initEnvironment(env)
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "skewt.h"

namespace skewt {

class Error : public std::runtime_error {
public:
    Error(skt_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    skt_status status;
};

class EnvironmentGPU {
public:
    EnvironmentGPU(int nx, int ny_vertical, int nz, float voxel, const skt_solver_cfg* cfg = nullptr) {
        skt_grid_desc g{nx, ny_vertical, nz, voxel};
        check(skt_create(&g, cfg, &env_), nullptr);
        n_ = size_t(nx) * ny_vertical * nz;
        grid_ = g;
    }
    ~EnvironmentGPU() { skt_destroy(env_); }
    EnvironmentGPU(const EnvironmentGPU&) = delete;
    EnvironmentGPU& operator=(const EnvironmentGPU&) = delete;

    // environmentGPU::init. velField is (u, v, w) per cell, like the reference's glm::vec3 array.
    void init(const float* potTemps, const float* velField, const float* Qv, const float* groundTemp, const float* groundPres,
              const float* pressures, const float* smallPressure, const int32_t* groundHeight, bool noise = true,
              uint32_t seed = 100) {
        check(skt_init(env_, potTemps, velField, Qv, groundTemp, groundPres, pressures, smallPressure, groundHeight,
                       noise ? SKT_INIT_NOISE : 0u, seed));
    }

    // environmentGPU::updateGPU. Returns false when the pressure solve hit its iteration cap
    // (the step is still done, as in the reference).
    bool updateGPU(float dt, float speed, int nsteps = 1) {
        const skt_status s = skt_step(env_, dt, speed, nsteps);
        if (s == SKT_NOT_CONVERGED) return false;
        check(s);
        return true;
    }

    // updateGPU without waiting (graph mode): the steps are queued; sync() collects them and
    // returns false when a pressure solve among them hit its iteration cap.
    void updateGPUAsync(float dt, float speed, int nsteps = 1) { check(skt_step_async(env_, dt, speed, nsteps)); }
    bool sync() {
        const skt_status s = skt_sync(env_);
        if (s == SKT_NOT_CONVERGED) return false;
        check(s);
        return true;
    }

    // environmentGPU::getParamArray
    float* getParamArray(skt_param type, skt_direction windDir = SKT_RIGHT) {
        float* p = nullptr;
        check(skt_field_device_ptr(env_, type, windDir, &p));
        return p;
    }

    // one field of editor::GPUSetEnv's readback
    std::vector<float> readField(skt_param type, skt_direction windDir = SKT_RIGHT) {
        std::vector<float> out(n_);
        check(skt_read_field(env_, type, windDir, out.data(), out.size()));
        return out;
    }

    // the per-step readback without waiting: the fields as they stand after the queued step are
    // written to dst[i] (n floats each; pinned buffers for overlap) while the next steps run;
    // the buffers must stay valid until readWait()
    void readFieldsAsync(const std::vector<skt_param>& params, const std::vector<skt_direction>& dirs, float* const* dst) {
        std::vector<int> p(params.begin(), params.end()), d(dirs.begin(), dirs.end());
        if (d.size() != p.size()) throw Error(SKT_INVALID_ARG, "one direction per field");
        check(skt_read_fields_async(env_, int(p.size()), p.data(), d.data(), dst, n_));
    }
    void readWait() { check(skt_read_wait(env_)); }

    skt_step_stats stats() {
        skt_step_stats s{};
        check(skt_stats(env_, &s));
        return s;
    }

    skt_env* handle() { return env_; }
    const skt_grid_desc& grid() const { return grid_; }

private:
    void check(skt_status s, const skt_env* e = reinterpret_cast<const skt_env*>(1)) {
        if (s == SKT_OK) return;
        throw Error(s, skt_last_error(e == reinterpret_cast<const skt_env*>(1) ? env_ : e));
    }
    skt_env* env_ = nullptr;
    size_t n_ = 0;
    skt_grid_desc grid_{};
};

// readTable (Game/readTable.h:50-92), reading side. The reference opens the archive with
// miniz_cpp::zip_file; here the caller's zip library answers member reads (skt_archive_read_fn).
class ReadTable {
public:
    ReadTable() = default;
    ~ReadTable() { skt_sounding_free(&data_); }
    ReadTable(const ReadTable&) = delete;
    ReadTable& operator=(const ReadTable&) = delete;

    // readTable::readKNMIFile (Game/readTable.cpp:27-132)
    void readKNMIFile(skt_archive_read_fn read, void* ctx) {
        skt_sounding_free(&data_);
        check(skt_sounding_read_knmi(read, ctx, &data_));
    }

    // readTable::readDWDFile (Game/readTable.cpp:134-354); file is the archive's path string
    void readDWDFile(const char* file, skt_archive_read_fn read, void* ctx) {
        skt_sounding_free(&data_);
        check(skt_sounding_read_dwd(file, read, ctx, &data_));
    }

    // readTable::initEnvironment (Game/readTable.cpp:364-474): interpolate onto env's grid and
    // call env.init with the result (flat ground).
    void initEnvironment(EnvironmentGPU& env, bool noise = true, uint32_t seed = 100) {
        const skt_grid_desc& g = env.grid();
        const size_t n = size_t(g.nx) * g.ny * g.nz, ng = size_t(g.nx) * g.nz;
        std::vector<float> theta(n), vel(3 * n), qv(n), gT(ng), gp(ng), p3d(n), pcol(g.ny);
        check(skt_sounding_to_init(&data_, &g, theta.data(), vel.data(), qv.data(), gT.data(), gp.data(), p3d.data(),
                                   pcol.data()));
        std::vector<int32_t> gh(ng, 0);
        env.init(theta.data(), vel.data(), qv.data(), gT.data(), gp.data(), p3d.data(), pcol.data(), gh.data(), noise, seed);
    }

    const skt_sounding& data() const { return data_; }

private:
    static void check(skt_status s) {
        if (s != SKT_OK) throw Error(s, skt_last_error(nullptr));
    }
    skt_sounding data_{};
};

}  // namespace skewt
