// Tetrahedron quality with the normalisation of the MeshQuality example:
// 7.348469 * volume / (area * longest edge), where the area term adds the
// faces (0,1,2) and (0,1,3) only (the example's effective computation).
{
   float   l2max = 0.f, area;
   float4  e;
   int     i, j;

   for(i=0;i<4;i++)
      for(j=i+1;j<4;j++)
      {
         e = VerCrd[i] - VerCrd[j];
         l2max = max(l2max, dot(e, e));
      }

   area = CalTriSrf(VerCrd[0], VerCrd[1], VerCrd[2]) + CalTriSrf(VerCrd[0], VerCrd[1], VerCrd[3]);
   qal  = 7.348469 * CalTetVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]) / (area * sqrt(l2max));
}
