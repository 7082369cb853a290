/* Mean-ratio quality of a tetrahedron in the GMlib dialect:
     q = 12 (3 |V|)^(2/3) / (sum of the six squared edge lengths),
   1 for the regular tet, towards 0 as it flattens, and negative when the
   orientation determinant det = (b - a) . ((c - a) x (d - a)) is not
   positive (3 |V| = |det| / 2).  VerCrd[4]: the vertices, read through
   TetVer; qal: one float per tet.  The library's native quality pass
   computes the same measure and takes the sign of near-flat tets from an
   FP64 determinant; this body keeps FP32 throughout. */
{
   float4 ab = VerCrd[1] - VerCrd[0], ac = VerCrd[2] - VerCrd[0], ad = VerCrd[3] - VerCrd[0];
   float4 bc = VerCrd[2] - VerCrd[1], bd = VerCrd[3] - VerCrd[1], cd = VerCrd[3] - VerCrd[2];
   float  det = dot(cross(ac, ad), ab);
   float  l2 = dot(ab, ab) + dot(ac, ac) + dot(ad, ad) + dot(bc, bc) + dot(bd, bd) + dot(cd, cd);
   float  q = 12.f * pow(.5f * fabs(det), 2.f / 3.f) / l2;

   qal = det > 0.f ? q : -q;
}
