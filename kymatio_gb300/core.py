"""Op-by-op scattering cascades over a backend object.

Restatements of kymatio's depth-first cores that only call the backend op
surface (pad, unpad, rfft, ifft, irfft, cdgmm, modulus, subsample_fourier,
stack).  Driven by ``kymatio_gb300.backend.backend2d`` / ``backend1d`` they
run every op as a CUDA kernel of this package; they are the op-level path
(one launch per op, as the reference's torch backend does), while the
``Scattering2D`` / ``Scattering1D`` modules run the fused cascade.
"""


def scattering2d(x, pad, unpad, backend, J, L, phi, psi, max_order, out_type='array'):
    """kymatio/scattering2d/core/scattering2d.py:1-88."""
    out_S_0, out_S_1, out_S_2 = [], [], []
    U_0_c = backend.rfft(pad(x))
    S_0 = unpad(backend.irfft(backend.subsample_fourier(backend.cdgmm(U_0_c, phi['levels'][0]), k=2 ** J)))
    out_S_0.append({'coef': S_0, 'j': (), 'n': (), 'theta': ()})
    for n1 in range(len(psi)):
        j1, theta1 = psi[n1]['j'], psi[n1]['theta']
        U_1_c = backend.cdgmm(U_0_c, psi[n1]['levels'][0])
        if j1 > 0:
            U_1_c = backend.subsample_fourier(U_1_c, k=2 ** j1)
        U_1_c = backend.rfft(backend.modulus(backend.ifft(U_1_c)))
        S_1_c = backend.subsample_fourier(backend.cdgmm(U_1_c, phi['levels'][j1]), k=2 ** (J - j1))
        out_S_1.append({'coef': unpad(backend.irfft(S_1_c)), 'j': (j1,), 'n': (n1,), 'theta': (theta1,)})
        if max_order < 2:
            continue
        for n2 in range(len(psi)):
            j2, theta2 = psi[n2]['j'], psi[n2]['theta']
            if j2 <= j1:
                continue
            U_2_c = backend.subsample_fourier(backend.cdgmm(U_1_c, psi[n2]['levels'][j1]), k=2 ** (j2 - j1))
            U_2_c = backend.rfft(backend.modulus(backend.ifft(U_2_c)))
            S_2_c = backend.subsample_fourier(backend.cdgmm(U_2_c, phi['levels'][j2]), k=2 ** (J - j2))
            out_S_2.append({'coef': unpad(backend.irfft(S_2_c)), 'j': (j1, j2), 'n': (n1, n2),
                            'theta': (theta1, theta2)})
    out_S = out_S_0 + out_S_1 + out_S_2
    if out_type == 'array':
        return backend.stack([s['coef'] for s in out_S])
    return out_S


def scattering1d(U_0, backend, filters, log2_stride, average_local):
    """kymatio/scattering1d/core/scattering1d.py:2-107 (generator of paths)."""
    U_0_hat = backend.rfft(U_0)
    phi = filters[0]
    if average_local:
        S_0 = backend.irfft(backend.subsample_fourier(backend.cdgmm(U_0_hat, phi['levels'][0]), 2 ** log2_stride))
        yield {'coef': S_0, 'j': (), 'n': ()}
    else:
        yield {'coef': U_0, 'j': (), 'n': ()}
    psi1 = filters[1]
    for n1 in range(len(psi1)):
        j1 = psi1[n1]['j']
        k1 = min(j1, log2_stride) if average_local else j1
        U_1_c = backend.ifft(backend.subsample_fourier(backend.cdgmm(U_0_hat, psi1[n1]['levels'][0]), 2 ** k1))
        U_1_m = backend.modulus(U_1_c)
        if average_local or len(filters) > 2:
            U_1_hat = backend.rfft(U_1_m)
        if average_local:
            k1_J = max(log2_stride - k1, 0)
            S_1 = backend.irfft(backend.subsample_fourier(backend.cdgmm(U_1_hat, phi['levels'][k1]), 2 ** k1_J))
            yield {'coef': S_1, 'j': (j1,), 'n': (n1,)}
        else:
            yield {'coef': U_1_m, 'j': (j1,), 'n': (n1,)}
        if len(filters) > 2:
            psi2 = filters[2]
            for n2 in range(len(psi2)):
                j2 = psi2[n2]['j']
                if j2 > j1:
                    sub2 = min(j2, log2_stride) if average_local else j2
                    k2 = max(sub2 - k1, 0)
                    U_2_c = backend.ifft(backend.subsample_fourier(backend.cdgmm(U_1_hat, psi2[n2]['levels'][k1]),
                                                                   2 ** k2))
                    U_2_m = backend.modulus(U_2_c)
                    if average_local:
                        U_2_hat = backend.rfft(U_2_m)
                        k2_T = max(log2_stride - sub2, 0)
                        S_2 = backend.irfft(backend.subsample_fourier(
                            backend.cdgmm(U_2_hat, phi['levels'][k1 + k2]), 2 ** k2_T))
                        yield {'coef': S_2, 'j': (j1, j2), 'n': (n1, n2)}
                    else:
                        yield {'coef': U_2_m, 'j': (j1, j2), 'n': (n1, n2)}
