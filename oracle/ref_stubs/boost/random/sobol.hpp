// Stand-in: lib/src/core.cpp:22-25 constructs a Sobol generator it never uses.
#pragma once
namespace boost { namespace random { struct sobol { explicit sobol(int) {} }; } }
