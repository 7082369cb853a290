// Mean of the optimal points of the ball (each tet contributes the point
// facing this vertex), then a 0.2 relaxation; res is the squared move.
{
   float4 acc = (float4)(0.);
   int    k;

   for(k=0;k<OptCrdDegMax;k++)
   {
      char s = VerTetVoy[k];
      acc += (s == 0) ? OptCrd[k][0] : (s == 1) ? OptCrd[k][1]
           : (s == 2) ? OptCrd[k][2] : OptCrd[k][3];
   }

   acc = acc * (float4)(1./(OptCrdDeg));
   acc = mix(VerCrd, acc, (float)0.2);
   res = dot(VerCrd - acc, VerCrd - acc);
   VerCrd = acc;
}
