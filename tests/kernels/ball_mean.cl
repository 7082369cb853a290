// Sum of a tetrahedron field over the vertex ball, divided by the degree.
{
   float4 s = (float4){0,0,0,0};
   for(int k=0;k<TetDatDegMax;k++)
      s += TetDat[k];
   VerDat = s / TetDatDeg;
}
