// Quality of the triangle (the toolkit's CalTriQal).
TriQ = CalTriQal(VerCrd[0], VerCrd[1], VerCrd[2]);
