// ORACLE — test infrastructure only. Stand-in for the game engine's core header, so that the
// reference's sounding reader (Game/readTable.cpp) compiles without the engine: it names only
// bee::Engine.DebugRenderer() (for its skew-T plot, which the tests never draw).
#pragma once
#include "rendering/debug_render.hpp"

namespace bee {
class EngineStub {
public:
    bee::DebugRenderer& DebugRenderer();
};
extern EngineStub Engine;
}  // namespace bee
