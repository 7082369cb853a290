TetDat = (VerCrd[0] + VerCrd[1] + VerCrd[2] + VerCrd[3]) * 0.25;
