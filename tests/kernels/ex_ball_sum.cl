// Sum of a tetrahedron field over the vertex ball (zero past the degree).
{
   float4 acc = (float4)(0.0f);
   for(int k = 0; k < CelDegMax; k++)
      acc += Cel[k];
   Pts = acc;
}
