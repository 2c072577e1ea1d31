/* Test infrastructure (oracle only): the fprintf replacement used by
 * oracle/_ref/NumCalc_dump.  Any %E / % E conversion that has no explicit
 * precision is printed with precision 16 (17 significant digits); all other
 * text and conversions pass through unchanged. */
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

int oracle_fprintf(FILE *f, const char *fmt, ...)
{
    char out[1024];
    size_t o = 0, n = strlen(fmt);
    for (size_t i = 0; i < n && o + 8 < sizeof(out); ++i) {
        out[o++] = fmt[i];
        if (fmt[i] != '%') continue;
        if (i + 1 < n && fmt[i + 1] == '%') { out[o++] = fmt[++i]; continue; }
        /* copy flags, then add a precision in front of E if none was given */
        size_t j = i + 1;
        while (j < n && strchr(" +-#0", fmt[j])) out[o++] = fmt[j++];
        if (j < n && (fmt[j] == 'E' || fmt[j] == 'e')) {
            memcpy(out + o, ".16", 3);
            o += 3;
        }
        i = j - 1;
    }
    out[o] = '\0';
    va_list ap;
    va_start(ap, fmt);
    int r = vfprintf(f, out, ap);
    va_end(ap);
    return r;
}
