#include "HepMC3/StandIn.h"
