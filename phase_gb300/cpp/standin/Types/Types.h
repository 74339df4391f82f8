// Stand-in for Phase's src/Types/Types.h (Types.h:7-10) so the plugin
// compiles outside a Phase tree.  Inside Phase the real header is used.
#pragma once
#include <cstddef>
#include <functional>
typedef double Scalar;
typedef std::size_t Label;
typedef std::size_t Size;
typedef int Index;
