// A vertex's own 4-item line rewritten from its items and the sum of a tet
// field over its ball; the high-degree twin launch starts at a line offset.
{
   float s = 0.0f;
   for(int k = 0; k < QDegMax; k++)
      s += Q[k];
   float4 t0 = V4[0], t1 = V4[1], t2 = V4[2], t3 = V4[3];
   V4[0] = t3 + (float4)(s);
   V4[1] = t0 + t1;
   V4[2] = t1 - t2;
   V4[3] = t2 + t0;
}
