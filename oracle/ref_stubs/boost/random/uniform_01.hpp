#pragma once
namespace boost { template <class T> struct uniform_01 {}; }
