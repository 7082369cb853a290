// Per tetrahedron: both items of a two-item vertex field summed over the
// four vertices, the vertex-coordinate sum scaled by their sum and
// normalised; the residual is the launch's line count over GmlPar->res.
{
   float4 f0 = Sol[0][0] + Sol[1][0] + Sol[2][0] + Sol[3][0];
   float4 f1 = Sol[0][1] + Sol[1][1] + Sol[2][1] + Sol[3][1];
   float4 m = (VerCrd[0] + VerCrd[1] + VerCrd[2] + VerCrd[3]) * (f0 + f1);
   Mid = m * rsqrt(dot(m, m));
   Rsd = (float)count.s0 / GmlPar->res;
}
