// Boost-free precompiled-header stand-in used only when the reference's
// sources are compiled as a CPU oracle.  It pulls in the standard headers the
// reference's own pch.h provides, minus boost, and then the reference macros.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cassert>
#include <iostream>
#include <fstream>
#include <sstream>
#include <functional>
#include <thread>
#include <string>
#include <vector>
#include <memory>
#include <atomic>
#include <mutex>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <chrono>
#include <regex>
#include <tuple>
#include <numeric>
#include <algorithm>
#include <boost/optional.hpp>
#include <lightmetrica/macros.h>
