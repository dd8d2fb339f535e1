// ORACLE — test infrastructure only. Stands in for the engine's logger (Engine/include/tools/log.hpp,
// which needs the engine's fmt set-up) when the reference's colour schemes are compiled alone:
// bee::colorScheme calls Log::Error only for a scheme whose two ends coincide.
#pragma once

namespace bee {
struct Log {
    template <typename... A>
    static void Error(const A&...) {}
};
}  // namespace bee
