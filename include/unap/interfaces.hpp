/* UNAP::interfaces: the processor-boundary coupling of a matrix
 * (src/matrix/interfaces/interfaces.hpp).  The GB300 library solves one
 * system per GPU, so a matrix has no interfaces to other ranks: the object
 * exists so that code setting or reading it compiles, and it is empty. */
#ifndef INTERFACES_HPP
#define INTERFACES_HPP

#include "unapVector.hpp"

namespace UNAP
{

class interfaces
{
public:
    interfaces() {}
    virtual ~interfaces() {}
    /* number of neighbouring processors */
    label size() const { return 0; }
};

}  // namespace UNAP

#endif
