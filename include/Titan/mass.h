// Titan/mass.h -- point mass with the public interface of Titan's Mass
// (include/Titan/mass.h:16-76 in the reference).  The object lives on the host;
// Simulation::get/set/getAll/setAll move its state to and from the device.
#ifndef TITAN_GB300_MASS_H
#define TITAN_GB300_MASS_H

#include <cstdint>
#include <vector>

#include "vec.h"

namespace titan {

// include/Titan/object.h:223-225
enum CONSTRAINT_TYPE { CONSTRAINT_PLANE, CONTACT_PLANE, BALL, DIRECTION };

struct LocalConstraint {
    CONSTRAINT_TYPE type;
    Vec vec;
    double num;
};

class Mass {
public:
    // The `fixed` argument is accepted and ignored, as in the reference
    // (src/mass.cu:42-55); use fix().
    Mass(const Vec &position, double mass = 0.1, bool fixed = false);

    double m;  // mass in kg
    double T;  // local time
    Vec pos;   // position in m
    Vec vel;   // velocity in m/s

    void setExternalForce(const Vec &v) { extern_force = v; }
    Vec acceleration() { return acc; }

    void addConstraint(CONSTRAINT_TYPE type, const Vec &vec, double num);
    void clearConstraints(CONSTRAINT_TYPE type);
    void clearConstraints();

    void setDrag(double C);  // truncated to int on the device, as the reference does
    void fix();
    void unfix();

private:
    Mass();
    Vec acc;
    Vec extern_force;
    bool valid = true;
    int ref_count = 0;
    std::vector<LocalConstraint> constraints;
    double drag_coefficient = 0.0;
    bool fixed = false;
    int64_t index = -1;  // slot in the device scene

    void decrementRefCount();

    friend class Simulation;
    friend class Spring;
    friend class Container;
    friend class Lattice;
    friend class Beam;
    friend class Cube;
};

}  // namespace titan

#endif
