// ORACLE — test infrastructure only (pins oracle/view.py; never part of the product).
//
// Runs the reference's own colour schemes: the statements of editor::setColors
// (Game/editor.cpp:53-112, extracted at build time by oracle/build_ref.py into the git-ignored
// oracle/_ref/setcolors_body.inc) fill a bee::colorScheme (Engine/source/rendering/colors.cpp,
// compiled unmodified beside this file), and rc_get_color returns what getColor gives for a
// value. The editor reaches the schemes through bee::Engine.DebugRenderer().GetColorScheme();
// this file supplies that one path and nothing else of the engine.
#include "rendering/colors.hpp"

#include <string>

namespace bee {
struct RefDebugRenderer {
    colorScheme scheme;
    colorScheme& GetColorScheme() { return scheme; }
};
struct RefEngine {
    RefDebugRenderer renderer;
    RefDebugRenderer& DebugRenderer() { return renderer; }
};
RefEngine Engine;
}  // namespace bee

namespace {
void ref_set_colors() {
#include "setcolors_body.inc"
}
bool g_ready = false;
}  // namespace

extern "C" {

// getColor(name, value) into rgb[3]; returns getColor's own return value (1 when it
// interpolated), or -1 for an unknown scheme.
int rc_get_color(const char* name, float value, float* rgb) {
    if (!g_ready) {
        ref_set_colors();
        g_ready = true;
    }
    glm::vec3 c(0.0f);
    int r;
    try {
        r = bee::Engine.DebugRenderer().GetColorScheme().getColor(std::string(name), value, c) ? 1 : 0;
    } catch (...) {
        return -1;
    }
    rgb[0] = c.x;
    rgb[1] = c.y;
    rgb[2] = c.z;
    return r;
}

}  // extern "C"
