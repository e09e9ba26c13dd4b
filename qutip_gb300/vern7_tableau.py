"""Verner 7(6) "most efficient" Runge-Kutta tableau with 7th-order dense output.
Coefficients are J. Verner's published table RKV76.IIa (efficient), given here as exact
IEEE-754 doubles in hex form so that every host and device consumer reads the same bits.
The reference loads the same table in qutip/solver/integrator/verner7efficient.py:10-333;
the error weights are e = b - bhat (verner7efficient.py:108-110).
"""
ORDER = 7
RK_STEP = 10
RK_EXTRA_STEP = 16
DENSEOUT_ORDER = 7

C = [
    float.fromhex('0x0.0p+0'),
    float.fromhex('0x1.47ae147ae147bp-8'),
    float.fromhex('0x1.be02468acf135p-4'),
    float.fromhex('0x1.4e81b4e81b4e8p-3'),
    float.fromhex('0x1.d26e978d4fdf4p-2'),
    float.fromhex('0x1.38119f5c18ee8p-1'),
    float.fromhex('0x1.c49ba5e353f7dp-1'),
    float.fromhex('0x1.d99999999999ap-1'),
    float.fromhex('0x1.0000000000000p+0'),
    float.fromhex('0x1.0000000000000p+0'),
    float.fromhex('0x1.0000000000000p+0'),
    float.fromhex('0x1.28f5c28f5c28fp-2'),
    float.fromhex('0x1.0000000000000p-3'),
    float.fromhex('0x1.0000000000000p-2'),
    float.fromhex('0x1.0f5c28f5c28f6p-1'),
    float.fromhex('0x1.947ae147ae148p-1'),
]

B = [
    float.fromhex('0x1.824c7fe71401bp-5'),
    float.fromhex('0x0.0p+0'),
    float.fromhex('0x0.0p+0'),
    float.fromhex('0x1.07af8f2c9ce02p-2'),
    float.fromhex('0x1.0c7562a9bdcdcp-2'),
    float.fromhex('0x1.37a025dab0159p-3'),
    float.fromhex('0x1.f9da53eb6a44ep-2'),
    float.fromhex('-0x1.2d5dcbdcea09dp-2'),
    float.fromhex('0x1.4d138cc3aa306p-4'),
    float.fromhex('0x0.0p+0'),
]

E = [
    float.fromhex('0x1.4dd7897422b60p-9'),
    float.fromhex('0x0.0p+0'),
    float.fromhex('0x0.0p+0'),
    float.fromhex('-0x1.3c7c7d0e25400p-7'),
    float.fromhex('0x1.5898171705ca4p-5'),
    float.fromhex('-0x1.11216681df170p-4'),
    float.fromhex('0x1.0f5eb708b4518p-2'),
    float.fromhex('-0x1.2d5dcbdcea09dp-2'),
    float.fromhex('0x1.4d138cc3aa306p-4'),
    float.fromhex('-0x1.4c842c994e2b1p-6'),
]

# A[i] lists the stage-i weights a[i, 0..i-1] (strictly lower triangular).
A = [
    [],
    [float.fromhex('0x1.47ae147ae147bp-8')],
    [float.fromhex('-0x1.13a8847ce7186p+0'), float.fromhex('0x1.2f88a8e59409ap+0')],
    [float.fromhex('0x1.4e81b4e81b4e8p-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.f5c28f5c28f5cp-4')],
    [float.fromhex('0x1.471fb9cddc9bdp-1'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.3a537b236d238p+1'), float.fromhex('0x1.22d95fa19ff87p+1')],
    [float.fromhex('-0x1.54ae9142bd52dp+1'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.59be93e7f0391p+3'), float.fromhex('-0x1.0b5344d4e2ef6p+3'), float.fromhex('0x1.a416f336399e6p-1')],
    [float.fromhex('0x1.8455e02ba6d50p+2'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.8b616076cbec0p+4'), float.fromhex('0x1.46d71d0ab3120p+4'), float.fromhex('-0x1.e7f9f82406e6ep+0'), float.fromhex('0x1.01948128a32f7p+0')],
    [float.fromhex('0x1.81bfdb75b2798p+3'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.8e09ccb12e37ep+5'), float.fromhex('0x1.4924a2cc6e376p+5'), float.fromhex('-0x1.1d8d7a71af007p+2'), float.fromhex('0x1.056b3a3a7fe6cp+1'), float.fromhex('-0x1.92d5cf70abb45p-4')],
    [float.fromhex('0x1.446bb241baabep+3'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.55210bed841c7p+5'), float.fromhex('0x1.1e1c582ab6be0p+5'), float.fromhex('-0x1.164601976fe88p+2'), float.fromhex('0x1.01432ab412663p+1'), float.fromhex('0x1.651e784ce7ec1p-2'), float.fromhex('-0x1.15f41b4722d81p-2')],
    [float.fromhex('-0x1.683d96681eb23p+5'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.76a78c7eacee8p+7'), float.fromhex('-0x1.340ec1faa9e18p+7'), float.fromhex('0x1.2908d1a693680p+4'), float.fromhex('-0x1.c91368e7b5080p+2'), float.fromhex('0x1.4f0e1437ed68dp+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0')],
    [float.fromhex('0x1.824c7fe71401bp-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.07af8f2c9ce02p-2'), float.fromhex('0x1.0c7562a9bdcdcp-2'), float.fromhex('0x1.37a025dab0159p-3'), float.fromhex('0x1.f9da53eb6a44ep-2'), float.fromhex('-0x1.2d5dcbdcea09dp-2'), float.fromhex('0x1.4d138cc3aa306p-4'), float.fromhex('0x0.0p+0')],
    [float.fromhex('0x1.ac9fc4869b571p-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.ccb71aa3486a2p-3'), float.fromhex('0x1.1dcc382fa4b24p-6'), float.fromhex('-0x1.f69ed7c067ba3p-8'), float.fromhex('0x1.1977f66d5c342p-5'), float.fromhex('-0x1.500b36cf71ed2p-5'), float.fromhex('0x1.a444a657368c3p-6'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.06dedd044d4dbp-6')],
    [float.fromhex('0x1.b29cebb4ac4bep-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.f384ffe16a5dbp-4'), float.fromhex('0x1.22c3a524d2189p-6'), float.fromhex('-0x1.36d145618630dp-11'), float.fromhex('0x1.12a7eb6485529p-7'), float.fromhex('-0x1.a7cfad5c3bb9ep-7'), float.fromhex('0x1.346a0e1ad479dp-7'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.5ed4af05e0aafp-8'), float.fromhex('-0x1.1111bb0e37b50p-4')],
    [float.fromhex('0x1.3e7f3dad06358p-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.3fdb90067de74p-9'), float.fromhex('-0x1.6d23618ff1da5p-10'), float.fromhex('-0x1.f182ab4a2dd67p-12'), float.fromhex('0x1.9b1ffdfe4aba5p-12'), float.fromhex('-0x1.a93f4881561f9p-12'), float.fromhex('0x1.a145b497f4431p-13'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.af1951b6d8104p-14'), float.fromhex('0x1.155a77d8c47f4p-5'), float.fromhex('0x1.73b0aa59bea8bp-3')],
    [float.fromhex('0x1.d4e24b7bccad1p-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.c801b19ce4d66p-3'), float.fromhex('0x1.f9a548822362fp-4'), float.fromhex('0x1.4832e1f9423e2p-5'), float.fromhex('-0x1.afb5b488f7168p-5'), float.fromhex('0x1.866da91fa26aep-5'), float.fromhex('-0x1.5e6fcbb083effp-6'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.f1df989c08f20p-7'), float.fromhex('0x1.edffff92ef618p-4'), float.fromhex('-0x1.7537d33814e17p-6'), float.fromhex('0x0.0p+0')],
    [float.fromhex('0x1.a4d6f952c61c8p-5'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.1535312363f2bp-1'), float.fromhex('0x1.66cf34f912137p-2'), float.fromhex('0x1.22acc8d2248aap-3'), float.fromhex('0x1.af338dbd33410p-4'), float.fromhex('-0x1.fd3eb7f4d4a2cp-6'), float.fromhex('-0x1.e516fe0e55e60p-8'), float.fromhex('0x0.0p+0'), float.fromhex('-0x1.a1fbf386451d3p-8'), float.fromhex('-0x1.62d37ef91259cp-3'), float.fromhex('-0x1.755009e2198bbp-3'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0')],
]

# BI[i] lists the dense-output polynomial coefficients of stage i (degree 1..7).
BI = [
    [float.fromhex('0x1.0000000000000p+0'), float.fromhex('-0x1.0d3a77ca2d93ep+3'), float.fromhex('0x1.0d677133b85dep+5'), float.fromhex('-0x1.1b34d43e5896cp+6'), float.fromhex('0x1.42967a583e9c3p+6'), float.fromhex('-0x1.798d991d3b03dp+5'), float.fromhex('0x1.64483320ef144p+3')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x1.1828522440e60p+3'), float.fromhex('-0x1.61d6b71b34551p+6'), float.fromhex('0x1.5ae6d9fec65d4p+8'), float.fromhex('-0x1.3aa1063e147c2p+9'), float.fromhex('0x1.08d6b43e0b8e2p+9'), float.fromhex('-0x1.4eb7bdca7c981p+7')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x1.1d3a789aa5d4fp+3'), float.fromhex('-0x1.683e47325c39ep+6'), float.fromhex('0x1.612e455d5e9cap+8'), float.fromhex('-0x1.4052e73e31357p+9'), float.fromhex('0x1.0da1df53c22e6p+9'), float.fromhex('-0x1.54c6b450287e5p+7')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x1.4b178b570cc78p+2'), float.fromhex('-0x1.a22b3ed0214edp+5'), float.fromhex('0x1.99f8849c46273p+7'), float.fromhex('-0x1.73d4a2fa86bccp+8'), float.fromhex('0x1.38fcf3b10740ap+8'), float.fromhex('-0x1.8b92554d012aep+6')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x1.0cb9ddb2032f9p+4'), float.fromhex('-0x1.53669ad4315e1p+7'), float.fromhex('0x1.4cbf33f1a1108p+9'), float.fromhex('-0x1.2dca7d29449edp+10'), float.fromhex('0x1.fc108809fe256p+9'), float.fromhex('-0x1.410f5d2e3899ep+8')],
    [float.fromhex('0x0.0p+0'), float.fromhex('-0x1.403121beaccfap+3'), float.fromhex('0x1.9466f4d2ff22bp+6'), float.fromhex('-0x1.8c79528065bbdp+8'), float.fromhex('0x1.6796e1f556099p+9'), float.fromhex('-0x1.2eaf1e030ed74p+9'), float.fromhex('0x1.7e8c7e042b752p+7')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x1.61e1faa3b854dp+1'), float.fromhex('-0x1.bef421e5258eep+4'), float.fromhex('0x1.b630f059868ccp+6'), float.fromhex('-0x1.8d6cf59a82d40p+7'), float.fromhex('0x1.4e885d27af6abp+7'), float.fromhex('-0x1.a6cd03d9065cdp+5')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0'), float.fromhex('0x0.0p+0')],
    [float.fromhex('0x0.0p+0'), float.fromhex('-0x1.15b680965799dp+1'), float.fromhex('0x1.60446310755ddp+4'), float.fromhex('-0x1.5b9b292e2a0f3p+6'), float.fromhex('0x1.3e72a1ad02855p+7'), float.fromhex('-0x1.0fec751141cabp+7'), float.fromhex('0x1.5e56d66e7bfeap+5')],
    [float.fromhex('0x0.0p+0'), float.fromhex('-0x1.38f6e8f400e45p+2'), float.fromhex('0x1.6c10b36fd109bp+4'), float.fromhex('-0x1.ec7c48165e27dp+4'), float.fromhex('-0x1.660a76a07b28ep+1'), float.fromhex('0x1.f5e94b5cf6383p+4'), float.fromhex('-0x1.f4fd5b4ab2f7dp+3')],
    [float.fromhex('0x0.0p+0'), float.fromhex('0x1.5b96e77d3f9a9p+3'), float.fromhex('-0x1.9458016611d76p+5'), float.fromhex('0x1.117c655bea6e1p+6'), float.fromhex('0x1.8da7244871f5ep+2'), float.fromhex('-0x1.16b8627ef19acp+6'), float.fromhex('0x1.16355d43c20b7p+5')],
    [float.fromhex('0x0.0p+0'), float.fromhex('-0x1.6bee869afb31bp+3'), float.fromhex('0x1.0594c7011b15dp+7'), float.fromhex('-0x1.e8a6b0e65e1d5p+8'), float.fromhex('0x1.a01b812a7268bp+9'), float.fromhex('-0x1.4c631d78571b5p+9'), float.fromhex('0x1.9395f46ce3a28p+7')],
    [float.fromhex('0x0.0p+0'), float.fromhex('-0x1.7adda79e244e5p+2'), float.fromhex('0x1.fa36e2bd53e32p+5'), float.fromhex('-0x1.096ec440dcb1dp+8'), float.fromhex('0x1.040ceb1fbc5d2p+9'), float.fromhex('-0x1.d3698002aa7aap+8'), float.fromhex('0x1.36c61095b90dfp+7')],
    [float.fromhex('0x0.0p+0'), float.fromhex('-0x1.4fbfa9622318cp+3'), float.fromhex('0x1.a56bea1c89392p+6'), float.fromhex('-0x1.99709376bf564p+8'), float.fromhex('0x1.6e6a6ceaf555ap+9'), float.fromhex('-0x1.2f26f87665888p+9'), float.fromhex('0x1.78195aa31d0cfp+7')],
]
