/*
 * cl2h.c -- embed an OpenCL-C kernel body in a C header as a string, the
 * build-time tool that the compile_cl() CMake macro runs (reference
 * utilities/cl2h.c, same command line and declaration):
 *
 *    cl2h source.cl destination.h name   ->   char *name = "..." ;
 *
 * The string holds a "\n", then the file line by line, each line ending in
 * "\n", then one more line (empty when the file ends with a newline), as
 * the reference's headers do.  Quotes and backslashes are escaped, so any
 * body round-trips exactly; the reference drops backslashes instead (a
 * macro line continuation becomes one joined line, the same program).
 */
#include <stdio.h>
#include <stdlib.h>

int main(int argc, char **argv)
{
   FILE *in, *out;
   int c, open_line = 0;

   if(argc != 4)
   {
      puts("Usage : cl2h source.cl destination.h procedure");
      return 1;
   }
   if(!(in = fopen(argv[1], "r")))
   {
      printf("Cannot open %s for reading\n", argv[1]);
      return 1;
   }
   if(!(out = fopen(argv[2], "w")))
   {
      printf("Cannot open %s for writing\n", argv[2]);
      fclose(in);
      return 1;
   }
   fprintf(out, "char *%s = \"\\n\" \\\n", argv[3]);
   while((c = fgetc(in)) != EOF)
   {
      if(!open_line)
      {
         fputc('"', out);
         open_line = 1;
      }
      if(c == '\n')
      {
         fputs("\\n\" \\\n", out);
         open_line = 0;
      }
      else if(c == '"' || c == '\\')
      {
         fputc('\\', out);
         fputc(c, out);
      }
      else if(c != '\r')
         fputc(c, out);
   }
   /* the last line, partial or empty, ends with "\n" like the others */
   if(!open_line)
      fputc('"', out);
   fputs("\\n\" \\\n", out);
   fputs("\n;\n", out);
   fclose(in);
   return fclose(out) == 0 ? 0 : 1;
}
