/*
 * gml_tables.c -- constant tables of the GMlib mesh model.
 *
 * These values are part of the reference's observable contract and are kept
 * identical: type sizes and names seen by generated kernels, the element node
 * counts, and the topology tables that decide link widths and the local
 * numbering of edges and faces (reference sources/gmlib3.c:164-358).  They
 * define which ball codes, edge lists and generated local names a mesh gets,
 * so a different value would change results, not just speed.
 */
#include "gml_internal.h"

/* byte sizes of the OpenCL types of enum opencl_type (cl_int ... cl_char16) */
const int GmlOclTypSiz[ GmlMaxOclTyp ] = {
   4, 8, 16, 32, 64,          /* int .. int16       */
   4, 8, 16, 32, 64,          /* float .. float16   */
   8, 16, 32, 64, 128,        /* double .. double16 */
   1, 2, 4, 8, 16 };          /* char .. char16     */

const char *GmlOclTypStr[ GmlMaxOclTyp ] = {
   "int", "int2", "int4", "int8", "int16",
   "float", "float2", "float4", "float8", "float16",
   "double", "double2", "double4", "double8", "double16",
   "char", "char2", "char4", "char8", "char16" };

const int GmlTypVecSiz[ GmlMaxOclTyp ] = {
   1,2,4,8,16, 1,2,4,8,16, 1,2,4,8,16, 1,2,4,8,16 };

const int GmlOclVecPow[5] = { GmlInt, GmlInt2, GmlInt4, GmlInt8, GmlInt16 };

/* vertices are float4, elements store their nodes in the next power of two */
const int GmlMshItmTyp[ GmlMaxEleTyp ] = {
   GmlFlt4, GmlInt2, GmlInt4, GmlInt4, GmlInt4, GmlInt8, GmlInt8, GmlInt8 };

const int GmlEleNmbNod[ GmlMaxEleTyp ] = { 0, 2, 3, 4, 4, 5, 6, 8 };
const int GmlMshTypDim[ GmlMaxEleTyp ] = { 0, 1, 2, 2, 3, 3, 3, 3 };

const char *GmlBalTypStr[ GmlMaxEleTyp ] = {
   "Ver", "Edg", "Tri", "Qad", "Tet", "Pyr", "Pri", "Hex" };

const char *GmlMshTypStr[ GmlMaxEleTyp ] = {
   "VerCrd", "EdgVer", "TriVer", "QadVer", "TetVer", "PyrVer", "PriVer", "HexVer" };

const char *GmlMshRefStr[ GmlMaxEleTyp ] = {
   "VerRef", "EdgRef", "TriRef", "QadRef", "TetRef", "PyrRef", "PriRef", "HexRef" };

/* base width of a link table [source type][destination type] */
const int GmlLenMatBas[ GmlMaxEleTyp ][ GmlMaxEleTyp ] = {
   {0,16, 8, 4,32,16,16, 8},
   {2, 0, 2, 2, 8, 8, 8, 4},
   {4, 4, 0, 0, 2, 2, 2, 0},
   {4, 4, 0, 0, 0, 2, 2, 2},
   {4, 8, 4, 0, 4, 4, 4, 0},
   {8, 8, 4, 1, 4, 8, 8, 1},
   {8,16, 2, 4, 2, 8, 8, 4},
   {8,16, 0, 8, 0, 8, 8, 8} };

/* maximum width of the high-degree extension of an uplink table */
const int GmlLenMatMax[ GmlMaxEleTyp ][ GmlMaxEleTyp ] = {
   {0,64,16, 8,64,32,32,16},
   {2, 0, 2, 2,16,16,16, 8},
   {4, 4, 0, 0, 2, 2, 2, 0},
   {4, 4, 0, 0, 0, 2, 2, 2},
   {4, 8, 4, 0, 4, 4, 4, 0},
   {8, 8, 4, 1, 4, 8, 8, 1},
   {8,16, 2, 4, 2, 8, 8, 4},
   {8,16, 0, 8, 0, 8, 8, 8} };

/* number of sub-entities of type [col] in one element of type [row] */
const int GmlNmbTpoLnk[ GmlMaxEleTyp ][ GmlMaxEleTyp ] = {
   {1, 1, 1, 1, 1, 1, 1, 1},
   {2, 2, 1, 1, 1, 1, 1, 1},
   {3, 3, 3, 0, 2, 2, 2, 0},
   {4, 4, 0, 4, 0, 2, 2, 2},
   {4, 6, 4, 0, 4, 4, 4, 0},
   {5, 8, 4, 1, 4, 5, 5, 1},
   {6, 9, 2, 3, 2, 5, 5, 3},
   {8,12, 0, 6, 0, 6, 6, 6} };

const int GmlNgbTyp[8]    = {-1,0,1,1,2,3,3,3};
const int GmlItmNmbVer[8] = {1,2,3,4,4,5,6,8};
const int GmlItmNmbEdg[8] = {0,1,3,4,6,8,9,12};
const int GmlItmNmbFac[8] = {0,0,1,1,4,5,5,6};

/* vertex count of each element face (3 triangle, 4 quadrilateral) */
const int GmlItmFacDeg[8][6] = {
{0,0,0,0,0,0}, {0,0,0,0,0,0}, {3,0,0,0,0,0}, {4,0,0,0,0,0},
{3,3,3,3,0,0}, {3,3,3,3,4,0}, {3,3,4,4,4,0}, {4,4,4,4,4,4} };

/* local node pairs of each element edge */
const int GmlItmEdgNod[8][12][2] = {
{ {0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0} },
{ {0,1},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0} },
{ {0,1},{1,2},{2,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0} },
{ {0,1},{1,2},{2,3},{3,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0} },
{ {0,1},{1,2},{2,0},{3,0},{3,1},{3,2},{0,0},{0,0},{0,0},{0,0},{0,0},{0,0} },
{ {0,1},{3,2},{0,3},{1,2},{0,4},{1,4},{2,4},{3,4},{0,0},{0,0},{0,0},{0,0} },
{ {0,1},{1,2},{2,0},{3,4},{4,5},{5,3},{0,3},{1,4},{2,5},{0,0},{0,0},{0,0} },
{ {0,1},{3,2},{7,6},{4,5},{0,3},{4,7},{5,6},{1,2},{0,4},{1,5},{2,6},{3,7} } };

/* local node lists of each element face */
const int GmlItmFacNod[8][6][4] = {
{ {0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0} },
{ {0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0} },
{ {0,1,2,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0} },
{ {0,1,2,3},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0},{0,0,0,0} },
{ {1,2,3,0},{2,0,3,0},{3,0,1,0},{0,2,1,0},{0,0,0,0},{0,0,0,0} },
{ {0,1,4,0},{1,2,4,0},{2,3,4,0},{3,0,4,0},{3,2,1,0},{0,0,0,0} },
{ {0,2,1,0},{3,4,5,0},{0,1,4,3},{1,2,5,4},{3,5,2,0},{0,0,0,0} },
{ {0,4,7,3},{1,2,6,5},{0,1,5,4},{3,7,6,2},{0,3,2,1},{4,5,6,7} } };
