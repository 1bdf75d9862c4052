// sin(j pi/128), cos(j pi/128) for j = 0..63: double-float pairs
// {sin hi, sin lo, cos hi, cos lo} and the third floats {sin lo2, cos lo2};
// written by gen_dfloat_trig_table.py.
#define MPGOS_DF_TRIG_TABLE_MAIN \
    {0.0f, 0.0f, 0x1p+0f, 0.0f}, \
    {0x1.92156p-6f, -0x1.0b933p-31f, 0x1.ffd886p-1f, 0x1.099a1ap-30f}, \
    {0x1.91f66p-5f, -0x1.de44fep-30f, 0x1.ff621ep-1f, 0x1.bcb6bep-28f}, \
    {0x1.2d520ap-4f, -0x1.a63cc2p-29f, 0x1.fe9cdap-1f, 0x1.a03108p-26f}, \
    {0x1.917a6cp-4f, -0x1.eb25eap-31f, 0x1.fd88dap-1f, 0x1.e89292p-28f}, \
    {0x1.f564e6p-4f, -0x1.2ad19ep-29f, 0x1.fc2648p-1f, -0x1.e3cc06p-26f}, \
    {0x1.2c8106p-3f, 0x1.d1cc28p-28f, 0x1.fa7558p-1f, -0x1.eeb5d2p-30f}, \
    {0x1.5e2144p-3f, 0x1.22cff2p-29f, 0x1.f8765p-1f, -0x1.63ad16p-27f}, \
    {0x1.8f8b84p-3f, -0x1.cb2cfap-30f, 0x1.f6297cp-1f, 0x1.feeb96p-26f}, \
    {0x1.c0b826p-3f, 0x1.4fc9ecp-28f, 0x1.f38f3ap-1f, 0x1.8c9cb2p-26f}, \
    {0x1.f19f98p-3f, -0x1.37a83ap-29f, 0x1.f0a7fp-1f, -0x1.1b73cap-27f}, \
    {0x1.111d26p-2f, 0x1.58fb3cp-29f, 0x1.ed740ep-1f, 0x1.da1258p-27f}, \
    {0x1.294062p-2f, 0x1.dab3ep-27f, 0x1.e9f416p-1f, -0x1.273a44p-26f}, \
    {0x1.4135cap-2f, -0x1.7d134p-27f, 0x1.e6288ep-1f, 0x1.891c22p-26f}, \
    {0x1.58f9a8p-2f, -0x1.4a9c04p-27f, 0x1.e2121p-1f, 0x1.3da1bap-27f}, \
    {0x1.708854p-2f, -0x1.e0b74cp-27f, 0x1.ddb13cp-1f, -0x1.2667b8p-26f}, \
    {0x1.87de2ap-2f, 0x1.abaa58p-28f, 0x1.d906bcp-1f, 0x1.e651a8p-26f}, \
    {0x1.9ef794p-2f, 0x1.d476c6p-29f, 0x1.d4134ep-1f, -0x1.d646d8p-26f}, \
    {0x1.b5d1p-2f, 0x1.3c2b98p-27f, 0x1.ced7bp-1f, -0x1.786712p-26f}, \
    {0x1.cc66eap-2f, -0x1.b38ee8p-28f, 0x1.c954b2p-1f, 0x1.3411f4p-29f}, \
    {0x1.e2b5d4p-2f, -0x1.fe4272p-28f, 0x1.c38b3p-1f, -0x1.cfe84ap-26f}, \
    {0x1.f8ba4ep-2f, -0x1.01d952p-28f, 0x1.bd7c0ap-1f, 0x1.8df2a6p-26f}, \
    {0x1.07387ap-1f, -0x1.b74004p-27f, 0x1.b72834p-1f, 0x1.465b9p-27f}, \
    {0x1.11eb36p-1f, -0x1.7c969cp-26f, 0x1.b090a6p-1f, -0x1.fabf8p-27f}, \
    {0x1.1c73b4p-1f, -0x1.9465cep-27f, 0x1.a9b662p-1f, 0x1.21d434p-26f}, \
    {0x1.26d054p-1f, 0x1.9ba25cp-26f, 0x1.a29a7ap-1f, 0x1.189e08p-31f}, \
    {0x1.30ff8p-1f, -0x1.8f47e6p-28f, 0x1.9b3e04p-1f, 0x1.fce1dp-27f}, \
    {0x1.3affa2p-1f, 0x1.240a18p-26f, 0x1.93a224p-1f, 0x1.324c8p-26f}, \
    {0x1.44cf32p-1f, 0x1.424776p-27f, 0x1.8bc806p-1f, 0x1.62a2e8p-26f}, \
    {0x1.4e6cacp-1f, -0x1.070686p-27f, 0x1.83b0ep-1f, 0x1.7ff2eep-26f}, \
    {0x1.57d694p-1f, -0x1.6e626cp-26f, 0x1.7b5df2p-1f, 0x1.3557d8p-28f}, \
    {0x1.610b76p-1f, -0x1.5c5a64p-26f, 0x1.72d084p-1f, -0x1.02000ep-26f}, \
    {0x1.6a09e6p-1f, 0x1.9fcef4p-27f, 0x1.6a09e6p-1f, 0x1.9fcef4p-27f}, \
    {0x1.72d084p-1f, -0x1.02000ep-26f, 0x1.610b76p-1f, -0x1.5c5a64p-26f}, \
    {0x1.7b5df2p-1f, 0x1.3557d8p-28f, 0x1.57d694p-1f, -0x1.6e626cp-26f}, \
    {0x1.83b0ep-1f, 0x1.7ff2eep-26f, 0x1.4e6cacp-1f, -0x1.070686p-27f}, \
    {0x1.8bc806p-1f, 0x1.62a2e8p-26f, 0x1.44cf32p-1f, 0x1.424776p-27f}, \
    {0x1.93a224p-1f, 0x1.324c8p-26f, 0x1.3affa2p-1f, 0x1.240a18p-26f}, \
    {0x1.9b3e04p-1f, 0x1.fce1dp-27f, 0x1.30ff8p-1f, -0x1.8f47e6p-28f}, \
    {0x1.a29a7ap-1f, 0x1.189e08p-31f, 0x1.26d054p-1f, 0x1.9ba25cp-26f}, \
    {0x1.a9b662p-1f, 0x1.21d434p-26f, 0x1.1c73b4p-1f, -0x1.9465cep-27f}, \
    {0x1.b090a6p-1f, -0x1.fabf8p-27f, 0x1.11eb36p-1f, -0x1.7c969cp-26f}, \
    {0x1.b72834p-1f, 0x1.465b9p-27f, 0x1.07387ap-1f, -0x1.b74004p-27f}, \
    {0x1.bd7c0ap-1f, 0x1.8df2a6p-26f, 0x1.f8ba4ep-2f, -0x1.01d952p-28f}, \
    {0x1.c38b3p-1f, -0x1.cfe84ap-26f, 0x1.e2b5d4p-2f, -0x1.fe4272p-28f}, \
    {0x1.c954b2p-1f, 0x1.3411f4p-29f, 0x1.cc66eap-2f, -0x1.b38ee8p-28f}, \
    {0x1.ced7bp-1f, -0x1.786712p-26f, 0x1.b5d1p-2f, 0x1.3c2b98p-27f}, \
    {0x1.d4134ep-1f, -0x1.d646d8p-26f, 0x1.9ef794p-2f, 0x1.d476c6p-29f}, \
    {0x1.d906bcp-1f, 0x1.e651a8p-26f, 0x1.87de2ap-2f, 0x1.abaa58p-28f}, \
    {0x1.ddb13cp-1f, -0x1.2667b8p-26f, 0x1.708854p-2f, -0x1.e0b74cp-27f}, \
    {0x1.e2121p-1f, 0x1.3da1bap-27f, 0x1.58f9a8p-2f, -0x1.4a9c04p-27f}, \
    {0x1.e6288ep-1f, 0x1.891c22p-26f, 0x1.4135cap-2f, -0x1.7d134p-27f}, \
    {0x1.e9f416p-1f, -0x1.273a44p-26f, 0x1.294062p-2f, 0x1.dab3ep-27f}, \
    {0x1.ed740ep-1f, 0x1.da1258p-27f, 0x1.111d26p-2f, 0x1.58fb3cp-29f}, \
    {0x1.f0a7fp-1f, -0x1.1b73cap-27f, 0x1.f19f98p-3f, -0x1.37a83ap-29f}, \
    {0x1.f38f3ap-1f, 0x1.8c9cb2p-26f, 0x1.c0b826p-3f, 0x1.4fc9ecp-28f}, \
    {0x1.f6297cp-1f, 0x1.feeb96p-26f, 0x1.8f8b84p-3f, -0x1.cb2cfap-30f}, \
    {0x1.f8765p-1f, -0x1.63ad16p-27f, 0x1.5e2144p-3f, 0x1.22cff2p-29f}, \
    {0x1.fa7558p-1f, -0x1.eeb5d2p-30f, 0x1.2c8106p-3f, 0x1.d1cc28p-28f}, \
    {0x1.fc2648p-1f, -0x1.e3cc06p-26f, 0x1.f564e6p-4f, -0x1.2ad19ep-29f}, \
    {0x1.fd88dap-1f, 0x1.e89292p-28f, 0x1.917a6cp-4f, -0x1.eb25eap-31f}, \
    {0x1.fe9cdap-1f, 0x1.a03108p-26f, 0x1.2d520ap-4f, -0x1.a63cc2p-29f}, \
    {0x1.ff621ep-1f, 0x1.bcb6bep-28f, 0x1.91f66p-5f, -0x1.de44fep-30f}, \
    {0x1.ffd886p-1f, 0x1.099a1ap-30f, 0x1.92156p-6f, -0x1.0b933p-31f}
#define MPGOS_DF_TRIG_TABLE_TAIL \
    {0.0f, 0.0f}, \
    {-0x1.0363acp-57f, -0x1.1354d4p-55f}, \
    {0x1.f376a2p-56f, 0x1.e3a844p-53f}, \
    {0x1.732fbcp-54f, -0x1.7ab784p-51f}, \
    {-0x1.e2718ep-60f, 0x1.9e0828p-53f}, \
    {-0x1.cbb1f8p-56f, 0x1.a3d90cp-52f}, \
    {-0x1.7768p-53f, -0x1.7a0a8cp-55f}, \
    {-0x1.ab3802p-55f, 0x1.3564acp-53f}, \
    {-0x1.49b466p-55f, 0x1.562172p-56f}, \
    {0x1.7e50ecp-54f, -0x1.cebdd8p-51f}, \
    {0x1.57a422p-54f, -0x1.ab4e14p-54f}, \
    {-0x1.3ed9fp-55f, 0x1.9e82c8p-52f}, \
    {0x1.6a2d72p-52f, -0x1.689f4ep-51f}, \
    {0x1.4325f2p-54f, 0x1.ee94aap-53f}, \
    {-0x1.80f7eep-53f, -0x1.a0298ep-52f}, \
    {-0x1.512c68p-54f, -0x1.cf879p-52f}, \
    {0x1.68d312p-53f, 0x1.8a2bf4p-51f}, \
    {-0x1.d24afep-54f, -0x1.94ef52p-51f}, \
    {0x1.5b362cp-57f, 0x1.786126p-52f}, \
    {-0x1.e97af2p-54f, 0x1.ed048ap-54f}, \
    {0x1.8f06c4p-53f, 0x1.a47d3ap-54f}, \
    {0x1.fb44f8p-54f, -0x1.9825a8p-51f}, \
    {-0x1.34b402p-52f, -0x1.378d3ep-52f}, \
    {0x1.421b8ap-52f, -0x1.926da4p-55f}, \
    {0x1.b25dd2p-55f, 0x1.819f64p-52f}, \
    {-0x1.5769dp-53f, -0x1.128bbp-56f}, \
    {0x1.c20674p-54f, 0x1.6788ecp-54f}, \
    {-0x1.b0e0eep-51f, -0x1.2c2be6p-51f}, \
    {-0x1.e7f896p-53f, 0x1.69d0f6p-54f}, \
    {0x1.13c294p-53f, -0x1.16f42p-52f}, \
    {-0x1.75720ap-55f, -0x1.21ea7p-53f}, \
    {-0x1.24a366p-53f, 0x1.90d4fp-51f}, \
    {-0x1.b7ba68p-52f, -0x1.b7ba68p-52f}, \
    {0x1.90d4fp-51f, -0x1.24a366p-53f}, \
    {-0x1.21ea7p-53f, -0x1.75720ap-55f}, \
    {-0x1.16f42p-52f, 0x1.13c294p-53f}, \
    {0x1.69d0f6p-54f, -0x1.e7f896p-53f}, \
    {-0x1.2c2be6p-51f, -0x1.b0e0eep-51f}, \
    {0x1.6788ecp-54f, 0x1.c20674p-54f}, \
    {-0x1.128bbp-56f, -0x1.5769dp-53f}, \
    {0x1.819f64p-52f, 0x1.b25dd2p-55f}, \
    {-0x1.926da4p-55f, 0x1.421b8ap-52f}, \
    {-0x1.378d3ep-52f, -0x1.34b402p-52f}, \
    {-0x1.9825a8p-51f, 0x1.fb44f8p-54f}, \
    {0x1.a47d3ap-54f, 0x1.8f06c4p-53f}, \
    {0x1.ed048ap-54f, -0x1.e97af2p-54f}, \
    {0x1.786126p-52f, 0x1.5b362cp-57f}, \
    {-0x1.94ef52p-51f, -0x1.d24afep-54f}, \
    {0x1.8a2bf4p-51f, 0x1.68d312p-53f}, \
    {-0x1.cf879p-52f, -0x1.512c68p-54f}, \
    {-0x1.a0298ep-52f, -0x1.80f7eep-53f}, \
    {0x1.ee94aap-53f, 0x1.4325f2p-54f}, \
    {-0x1.689f4ep-51f, 0x1.6a2d72p-52f}, \
    {0x1.9e82c8p-52f, -0x1.3ed9fp-55f}, \
    {-0x1.ab4e14p-54f, 0x1.57a422p-54f}, \
    {-0x1.cebdd8p-51f, 0x1.7e50ecp-54f}, \
    {0x1.562172p-56f, -0x1.49b466p-55f}, \
    {0x1.3564acp-53f, -0x1.ab3802p-55f}, \
    {-0x1.7a0a8cp-55f, -0x1.7768p-53f}, \
    {0x1.a3d90cp-52f, -0x1.cbb1f8p-56f}, \
    {0x1.9e0828p-53f, -0x1.e2718ep-60f}, \
    {-0x1.7ab784p-51f, 0x1.732fbcp-54f}, \
    {0x1.e3a844p-53f, 0x1.f376a2p-56f}, \
    {-0x1.1354d4p-55f, -0x1.0363acp-57f}
