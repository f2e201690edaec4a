// Titan/spring.h -- Hooke spring with the public interface of Titan's Spring
// (include/Titan/spring.h:17-66 in the reference), including the actuation
// fields _type/_omega/_damping.  _amplitude and _phase extend the reference's
// fixed 1 -/+ 0.2 sin(omega t) actuation; their defaults reproduce it.
#ifndef TITAN_GB300_SPRING_H
#define TITAN_GB300_SPRING_H

#include <cstdint>

#include "mass.h"
#include "vec.h"

namespace titan {

enum SpringType { PASSIVE_SOFT, PASSIVE_STIFF, ACTIVE_CONTRACT_THEN_EXPAND, ACTIVE_EXPAND_THEN_CONTRACT };

class Spring {
public:
    Spring() : _left(nullptr), _right(nullptr), _k(10000.0), _rest(1.0), _type(PASSIVE_SOFT), _omega(0.0), _damping(0.0) {}
    Spring(Mass *left, Mass *right)
        : _left(left), _right(right), _k(10000.0), _rest(1.0), _type(PASSIVE_SOFT), _omega(0.0), _damping(0.0) {
        defaultLength();
    }
    Spring(Mass *left, Mass *right, double k, double rest_length)
        : _left(left), _right(right), _k(k), _rest(rest_length), _type(PASSIVE_SOFT), _omega(0.0), _damping(0.0) {}
    Spring(Mass *left, Mass *right, double k, double rest_length, SpringType type, double omega)
        : _left(left), _right(right), _k(k), _rest(rest_length), _type(type), _omega(omega), _damping(0.0) {}

    void setRestLength(double rest_length) { _rest = rest_length; }
    void defaultLength() { _rest = (_left->pos - _right->pos).norm(); }
    void changeType(SpringType type, double omega) {
        _type = type;
        _omega = omega;
    }
    void addDamping(double constant) { _damping = constant; }
    void setActuation(double amplitude, double phase) {
        _amplitude = amplitude;
        _phase = phase;
    }

    void setLeft(Mass *left);
    void setRight(Mass *right);
    void setMasses(Mass *left, Mass *right) {
        _left = left;
        _right = right;
    }

    Mass *_left;
    Mass *_right;
    double _k;     // N/m
    double _rest;  // m
    SpringType _type;
    double _omega;    // rad/s
    double _damping;  // N s/m
    double _amplitude = 0.2;  // extension: rest-length modulation amplitude
    double _phase = 0.0;      // extension: modulation phase (rad)

private:
    int64_t index = -1;
    friend class Simulation;
    friend class Container;
    friend class Lattice;
    friend class Cube;
    friend class Beam;
};

}  // namespace titan

#endif
