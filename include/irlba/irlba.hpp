// CppIrlba's umbrella header name (include/irlba/irlba.hpp), forwarding to the
// GB300 engine's drop-in so a caller's `#include "irlba/irlba.hpp"` keeps
// working with only the include path changed.
#ifndef IRLBA_GB300_FORWARD_IRLBA_HPP
#define IRLBA_GB300_FORWARD_IRLBA_HPP
#include "../irlba_gb300/irlba.hpp"
#endif
