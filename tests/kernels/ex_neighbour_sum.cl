// Sum of a tetrahedron field over the four face neighbours (the null value
// where a face is on the boundary).
NbSum = Mid[0] + Mid[1] + Mid[2] + Mid[3];
