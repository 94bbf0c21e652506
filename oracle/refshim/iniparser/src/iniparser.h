/* Stand-in for iniparser's header (parameter.c includes it as
 * <../iniparser/src/iniparser.h>; the library is not part of the reference
 * checkout).  Used only to compile the reference's parameter.c in place as a
 * test oracle.  The functions are implemented in files_glue.c. */
#ifndef REFSHIM_INIPARSER_H
#define REFSHIM_INIPARSER_H
typedef struct refshim_dict dictionary;
dictionary *iniparser_load(const char *path);
int iniparser_getint(dictionary *d, const char *key, int notfound);
double iniparser_getdouble(dictionary *d, const char *key, double notfound);
char *iniparser_getstring(dictionary *d, const char *key, char *def);
void iniparser_freedict(dictionary *d);
#endif
