// Sum of the four vertex coordinates of the tetrahedron, in node order.
Cel = VerCrd[0] + VerCrd[1] + VerCrd[2] + VerCrd[3];
