// Oracle test infrastructure: standard headers that the reference sources use without
// including them. MSVC's standard library (the reference's toolchain, CMakeLists.txt:17)
// pulls these in transitively; libstdc++ does not. Passed with -include to the oracle
// build only.
#pragma once
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <future>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <memory_resource>
#include <mutex>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>
