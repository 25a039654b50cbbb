#pragma once

struct Medium
{
    float ior;  ///< index of refraction

    static const Medium air;
};

inline const Medium Medium::air{1.0003f};
