// ORACLE — test infrastructure only. The reference's engine headers were written against MSVC's
// standard headers, which pull in <vector> and <algorithm> transitively; libstdc++ does not, so
// the reference's colour-scheme files are compiled with these two forced in first.
#pragma once
#include <algorithm>
#include <vector>
