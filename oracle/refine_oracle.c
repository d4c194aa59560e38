/* CPU oracle of the model refinement (TEST INFRASTRUCTURE ONLY: used by the
 * tests and never by the product library).
 *
 * A plain-C restatement of jif3D's ModelRefiner (ModelBase/ModelRefiner.cpp):
 * the axis refinement, and the projection of values and combination of
 * gradients with the reference's own index walk (FindEnd, re-run for every
 * y and z cell as the reference does).  Pinned against the reference's
 * test_ModelRefiner.cpp cases in tests/test_oracle.py.
 */
#include <stdlib.h>

/* RefineOneAxis, ModelRefiner.cpp:17-72.  Returns the number of refined
 * cells written to out (capacity ncoarse + nref), or -1 when the last cell
 * would not have a positive size (the reference throws FatalException). */
int orc_refine_axis(int ncoarse, const double *old_coords, const double *old_sizes, int nref_in,
                    const double *ref_coords, double *out)
{
    const size_t nold = (size_t)ncoarse;     /* OldCoordinates.size() - 1 (:24) */
    const size_t nref = (size_t)nref_in - 1; /* RefCoordinates.size() - 1 (:25) */
    double *temp = malloc(sizeof(double) * (nold + nref + 1));
    size_t ntemp = 0, refineindex = 0;
    for (size_t i = 0; i < nold; ++i) {
        temp[ntemp++] = old_coords[i];                                    /* :32 */
        if (refineindex < nref && ref_coords[refineindex] == old_coords[i]) /* :35-38 */
            ++refineindex;
        const double limit = old_coords[i] + old_sizes[i];                /* :40 */
        while (refineindex < nref && ref_coords[refineindex] < limit)     /* :43-48 */
            temp[ntemp++] = ref_coords[refineindex++];
    }
    /* adjacent_difference + rotate (:53-55): out[k] = temp[k+1] - temp[k] */
    for (size_t k = 0; k + 1 < ntemp; ++k)
        out[k] = temp[k + 1] - temp[k];
    double lastsize = old_sizes[nold - 1];                                /* :58-62 */
    if (refineindex > 0)
        lastsize += old_coords[nold - 1] - temp[ntemp - 1];
    free(temp);
    if (!(lastsize > 0.0))                                                /* :63-71 */
        return -1;
    out[ntemp - 1] = lastsize;
    return (int)ntemp;
}

/* FindEnd, ModelRefiner.cpp:92-102 */
static size_t find_end(size_t startindex, double cellsize, const double *new_sizes, size_t nnew)
{
    double currsize = 0.0;
    size_t endindex = startindex;
    while (currsize < cellsize && endindex < nnew) {
        currsize += new_sizes[endindex];
        ++endindex;
    }
    return endindex;
}

/* ProjectValues (mode 0, ModelRefiner.cpp:124-168) and CombineGradient
 * (mode 1, :170-218) over the same walk; fine is [fnx][fny][fnz], coarse
 * [cnx][cny][cnz], both z fastest. */
static void walk(int mode, int cnx, int cny, int cnz, const double *cxs, const double *cys,
                 const double *czs, int fnx, int fny, int fnz, const double *fxs,
                 const double *fys, const double *fzs, double *coarse, double *fine)
{
    size_t startx = 0, endx, starty = 0, endy, startz = 0, endz;
    for (int i = 0; i < cnx; ++i) {
        endx = find_end(startx, cxs[i], fxs, (size_t)fnx);
        for (int j = 0; j < cny; ++j) {
            endy = find_end(starty, cys[j], fys, (size_t)fny);
            for (int k = 0; k < cnz; ++k) {
                endz = find_end(startz, czs[k], fzs, (size_t)fnz);
                const size_t c = ((size_t)i * cny + j) * cnz + k;
                double result = 0.0; /* CombineValues :114-122 */
                for (size_t a = startx; a < endx; ++a)
                    for (size_t b = starty; b < endy; ++b)
                        for (size_t d = startz; d < endz; ++d) {
                            const size_t f = (a * fny + b) * fnz + d;
                            if (mode == 0)
                                fine[f] = coarse[c]; /* AssignValue :104-111 */
                            else
                                result += fine[f];
                        }
                if (mode == 1)
                    coarse[c] = result;
                startz = endz;
            }
            starty = endy;
            startz = 0;
        }
        startx = endx;
        starty = 0;
    }
}

void orc_refine_project(int cnx, int cny, int cnz, const double *cxs, const double *cys,
                        const double *czs, int fnx, int fny, int fnz, const double *fxs,
                        const double *fys, const double *fzs, const double *coarse, double *fine)
{
    walk(0, cnx, cny, cnz, cxs, cys, czs, fnx, fny, fnz, fxs, fys, fzs, (double *)coarse, fine);
}

void orc_refine_combine(int cnx, int cny, int cnz, const double *cxs, const double *cys,
                        const double *czs, int fnx, int fny, int fnz, const double *fxs,
                        const double *fys, const double *fzs, const double *fine, double *coarse)
{
    walk(1, cnx, cny, cnz, cxs, cys, czs, fnx, fny, fnz, fxs, fys, fzs, coarse, (double *)fine);
}
