// Cell-centred heat flow, explicit Euler step.
SolTet += GmlPar->dt * Rhs;
