#pragma once

// First-hit debug views (include/DebugOptions.hpp); values equal dr_debug_view.
enum class DebugOptions : int {
    Off = 0,
    UVChecker = 1,
    BariCoords = 2,
    WindingOrder = 3,
};
