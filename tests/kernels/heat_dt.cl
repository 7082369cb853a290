// Cell-centred heat flow, stable time step of a cell: 0.3 V^(2/3).
dt = 0.3f * pow(CalTetVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]), 2.f / 3.f);
