#pragma once
namespace boost { template <class E, class D> struct variate_generator { variate_generator(E, D) {} }; }
