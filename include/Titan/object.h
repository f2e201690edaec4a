// Titan/object.h -- containers of masses and springs with the interface of
// Titan's Container / Cube / Lattice / Beam (include/Titan/object.h:230-285 in
// the reference).  The lattice geometry and spring order are those of
// src/object.cu:232-293, which define the mass and spring numbering.
#ifndef TITAN_GB300_OBJECT_H
#define TITAN_GB300_OBJECT_H

#include <vector>

#include "mass.h"
#include "spring.h"
#include "vec.h"

namespace titan {

class Container {
public:
    virtual ~Container() {}
    void translate(const Vec &displ);
    void rotate(const Vec &axis, double angle);  // radians, about the centre of mass
    void setMassValues(double m);                // adds m to every mass (src/object.cu:143-147)
    void setSpringConstants(double k);
    void setRestLengths(double len);
    void addConstraint(CONSTRAINT_TYPE type, const Vec &v, double d);
    void clearConstraints();
    void fix();

    void add(Mass *m);
    void add(Spring *s);
    void add(Container *c);

    std::vector<Mass *> masses;
    std::vector<Spring *> springs;
};

class Cube : public Container {
public:
    ~Cube() {}
    Cube(const Vec &center, double side_length = 1.0);
    double _side_length;
    Vec _center;
};

class Lattice : public Container {
public:
    ~Lattice() {}
    Lattice(const Vec &center, const Vec &dims, int nx = 10, int ny = 10, int nz = 10);
    int nx, ny, nz;
    Vec _center, _dims;
};

class Beam : public Container {
public:
    ~Beam() {}
    Beam(const Vec &center, const Vec &dims, int nx = 10, int ny = 10, int nz = 10);  // i == 0 face fixed
    int nx, ny, nz;
    Vec _center, _dims;
};

}  // namespace titan

#endif
