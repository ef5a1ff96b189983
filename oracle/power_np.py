"""Restatement of fastpm/utils.py:77-164 ``power`` — TEST INFRASTRUCTURE ONLY.

Integer-shell P(k): shell d = floor(sqrt(nx^2 + ny^2 + nz^2)) (find_root,
utils.py:125-133, restated with the same refinement loop), Hermitian weight 2 on the r2c half axis except its first and
last planes (147-149), k = sum(|n| 2pi/L w) / sum(w), P = sum(|f1 f2*| w) / sum(w)
L^3 (153-164).  A field whose k=0 mode is non-zero is first divided by
|f[0,0,0]| (95-96), so a density (1 + delta) field is normalised by its mean.
"""
import numpy


def power(f1, f2=None, boxsize=1.0, average=True):
    def tocomplex(f):
        f = numpy.asarray(f)
        return f if f.dtype.kind == 'c' else numpy.fft.rfftn(f)

    f1 = tocomplex(f1).astype('c16')
    if f1[0, 0, 0] != 0.0:
        f1 = f1 / abs(f1[0, 0, 0])
    if f2 is None:
        f2 = f1
    else:
        f2 = tocomplex(f2).astype('c16')
        if f2[0, 0, 0] != 0.0:
            f2 = f2 / abs(f2[0, 0, 0])

    N0, N1, N2c = f1.shape
    n0 = numpy.arange(N0)
    n0[n0 > N0 // 2] -= N0
    n1 = numpy.arange(N1)
    n1[n1 > N1 // 2] -= N1
    n2 = numpy.arange(N2c)
    nb = N0 // 2
    ksum = numpy.zeros(nb)
    wsum = numpy.zeros(nb)
    xsum = numpy.zeros(nb)
    w = numpy.full(N2c, 2.0, dtype='f4')
    w[0] = 1
    w[-1] = 1
    w = numpy.broadcast_to(w, (N1, N2c))
    for i in range(N0):
        kk = n0[i] ** 2 + n1[:, None] ** 2 + n2[None, :] ** 2
        # find_root (utils.py:125-133): the first test is strict, but the loop
        # re-tests every mode with <=, so all modes end in floor(sqrt(n^2)).
        d = numpy.int64(numpy.sqrt(kk) - 2).clip(0)
        mask = (d + 1) ** 2 < kk
        while mask.any():
            d[mask] += 1
            mask = (d + 1) ** 2 <= kk
        xw = abs(f1[i] * f2[i].conjugate()) * w
        kw = kk ** 0.5 * 2 * numpy.pi / boxsize * w
        ksum += numpy.bincount(d.ravel(), weights=kw.ravel(), minlength=N0)[:nb]
        wsum += numpy.bincount(d.ravel(), weights=w.ravel(), minlength=N0)[:nb]
        xsum += numpy.bincount(d.ravel(), weights=xw.ravel(), minlength=N0)[:nb]
    with numpy.errstate(invalid='ignore', divide='ignore'):
        center = ksum / wsum
        if not average:
            return center, xsum * boxsize ** 3, wsum
        return center, xsum / wsum * boxsize ** 3
