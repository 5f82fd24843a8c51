/*
 * btVector3.h -- stand-in for Bullet's vector type so that the reference's
 * mesh/icospheremesh.cpp and its scene samplers compile for the oracle without Bullet (not
 * in this image).
 * TEST INFRASTRUCTURE: built only by oracle/build_ref.sh into oracle/_ref/.
 * Single-precision components; length() = sqrt(x*x + y*y + z*z) summed left to right and
 * normalized() multiplies by the reciprocal of the length, the order of Bullet's scalar
 * (non-SSE) code path.
 */
#pragma once
#include <cmath>

class btVector3 {
   public:
    btVector3() : v_{0.f, 0.f, 0.f} {}
    btVector3(const float& x, const float& y, const float& z) : v_{x, y, z} {}
    float x() const { return v_[0]; }
    float y() const { return v_[1]; }
    float z() const { return v_[2]; }
    float getX() const { return v_[0]; }
    float getY() const { return v_[1]; }
    float getZ() const { return v_[2]; }
    btVector3 operator+(const btVector3& o) const { return btVector3(v_[0] + o.v_[0], v_[1] + o.v_[1], v_[2] + o.v_[2]); }
    btVector3 operator-(const btVector3& o) const { return btVector3(v_[0] - o.v_[0], v_[1] - o.v_[1], v_[2] - o.v_[2]); }
    btVector3 operator*(const float& s) const { return btVector3(v_[0] * s, v_[1] * s, v_[2] * s); }
    float length() const { return std::sqrt(v_[0] * v_[0] + v_[1] * v_[1] + v_[2] * v_[2]); }
    btVector3 normalized() const {
        const float inv = 1.0f / length();
        return *this * inv;
    }

   private:
    float v_[3];
};

inline btVector3 operator*(const float& s, const btVector3& v) { return v * s; }
