// Minimum of a per-tetrahedron scalar over the vertex ball (runtime degree).
{
   vq = tq[0];
   for(int k=1;k<tqDeg;k++)
      vq = min(vq, tq[k]);
}
