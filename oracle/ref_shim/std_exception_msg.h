// Force-included (only) when compiling the reference's Perturbation1DImpl.cpp,
// which throws std::exception("...") -- a constructor only MSVC's library
// provides.  Every standard header that file reaches is included first, so the
// macro below rewrites only the reference's own call into std::runtime_error.
#pragma once
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <exception>
#include <execution>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>
#define exception(msg) runtime_error(msg)
