/* Generated by gen_voigt_table.py -- do not edit.
 * Real-axis Faddeeva data at x_j = j/10: {exp(-x^2), 2/sqrt(pi) F(x),
 * 2/sqrt(pi) (1 - 2 x F(x))}, F = Dawson's integral. */
#pragma once
#define FSG_VTAB_N 81
#define FSG_VTAB_H 0.1
#define FSG_VTAB_INVH 10.0
/* rows padded to 4 doubles (32 bytes) for two aligned 16-byte loads */
#define FSG_VTAB_INIT { \
    {0x1.0000000000000p+0, 0x0.0p+0, 0x1.20dd750429b6dp+0, 0.0}, \
    {0x1.fae7cfd2b9cfep-1, 0x1.cb1d7bbb2a4e0p-4, 0x1.1b2049de9f95dp+0, 0.0}, \
    {0x1.ebec97e700b8dp-1, 0x1.c20ddd90bb7efp-3, 0x1.0a5cc389b9f08p+0, 0.0}, \
    {0x1.d3eec9cf11a26p-1, 0x1.4691d52ebdd5dp-2, 0x1.dfc25d471a7a5p-1, 0.0}, \
    {0x1.b44c30d232e50p-1, 0x1.9fe680135e736p-2, 0x1.9b5eb6cd60d91p-1, 0.0}, \
    {0x1.8ebef9eac820bp-1, 0x1.ea6b5c4b5d507p-2, 0x1.4c853be2a4c57p-1, 0.0}, \
    {0x1.6535d4d756470p-1, 0x1.1248f65a881a1p-1, 0x1.f12d1e6a93699p-2, 0.0}, \
    {0x1.39aa2aaf607f6p-1, 0x1.26eefeece764cp-1, 0x1.49a570ac855abp-2, 0.0}, \
    {0x1.0df945c9630cep-1, 0x1.336943c42b0d5p-1, 0x1.577d29a03a2e4p-3, 0.0}, \
    {0x1.c788df7728475p-2, 0x1.38648a243dcccp-1, 0x1.ed8af8e2ec6ffp-6, 0.0}, \
    {0x1.78b56362cef38p-2, 0x1.36dd5ff434d34p-1, -0x1.5ffeaf00b1c70p-4, 0.0}, \
    {0x1.315aa0aba1522p-2, 0x1.30016588081dcp-1, -0x1.6c53d558934f5p-3, 0.0}, \
    {0x1.e53a61786f313p-3, 0x1.251133065cdcbp-1, -0x1.f68641b560f66p-3, 0.0}, \
    {0x1.79e55f482fdfep-3, 0x1.1745f7cb1f128p-1, -0x1.28c2ce0f9451ep-2, 0.0}, \
    {0x1.207a6139c6d76p-3, 0x1.07bcecbc68bffp-1, -0x1.4178f341a3bdep-2, 0.0}, \
    {0x1.afb718e8457f7p-4, 0x1.eed3252df3b5dp-2, -0x1.49039b7934462p-2, 0.0}, \
    {0x1.3ca3e54079d1ap-4, 0x1.ce1d5a2b48277p-2, -0x1.434e7fad0cd62p-2, 0.0}, \
    {0x1.c747c3f342753p-5, 0x1.ae7a3f12078e7p-2, -0x1.3429cf2ca6090p-2, 0.0}, \
    {0x1.40d4a4144abecp-5, 0x1.90aea1cdb687cp-2, -0x1.1efed8d3ea40ap-2, 0.0}, \
    {0x1.bb37ab65978dcp-6, 0x1.752f1a2ee2788p-2, -0x1.06a38f6e4f551p-2, 0.0}, \
    {0x1.2c155b8213cf4p-6, 0x1.5c2fd528534ddp-2, -0x1.da9301214cb7cp-3, 0.0}, \
    {0x1.8e4d06b3b756bp-7, 0x1.45b4f3e9d855cp-2, -0x1.a90458be31e6bp-3, 0.0}, \
    {0x1.03192d479714bp-7, 0x1.31a1b558272a1p-2, -0x1.7aa360800aef1p-3, 0.0}, \
    {0x1.4a6ab36dfd3abp-8, 0x1.1fc552e382220p-2, -0x1.50921f3ef91bep-3, 0.0}, \
    {0x1.9d05c285d1a76p-9, 0x1.0fe517423f71ap-2, -0x1.2b45372779bf9p-3, 0.0}, \
    {0x1.fa0e9586aebc7p-10, 0x1.01c3ae396eba0p-2, -0x1.0ab9261d058d8p-3, 0.0}, \
    {0x1.2fe28d8fdc6e6p-10, 0x1.ea4bf74ceaebep-3, -0x1.dd3ebbaa22f50p-4, 0.0}, \
    {0x1.65bc855fb506ep-11, 0x1.d3abe1b6a5966p-3, -0x1.ad029bd860eaep-4, 0.0}, \
    {0x1.9ccaba7b2182dp-12, 0x1.bf47c48146c3dp-3, -0x1.83b2e23216bdcp-4, 0.0}, \
    {0x1.d2e37e8beae93p-13, 0x1.accdabbc2aab6p-3, -0x1.604744aa86bd8p-4, 0.0}, \
    {0x1.02cf22526545ap-13, 0x1.9bf85e103884fp-3, -0x1.41cd18800acdep-4, 0.0}, \
    {0x1.193f91c13e22fp-14, 0x1.8c8e066f90559p-3, -0x1.277032be62513p-4, 0.0}, \
    {0x1.2b94c2b893416p-15, 0x1.7e5e99b97fd56p-3, -0x1.107d2c36fc0b1p-4, 0.0}, \
    {0x1.38ca437a902c0p-16, 0x1.71423aeeedc93p-3, -0x1.f8bf7351b517ap-5, 0.0}, \
    {0x1.401d6005081c8p-17, 0x1.6517c2ec8a9eap-3, -0x1.d53e1569839abp-5, 0.0}, \
    {0x1.411fb0da07713p-18, 0x1.59c37c104e687p-3, -0x1.b5b2f1435c92fp-5, 0.0}, \
    {0x1.3bc1de4d1002cp-19, 0x1.4f2e153ea7ea5p-3, -0x1.99809020e04e3p-5, 0.0}, \
    {0x1.305522bf9aeb9p-20, 0x1.4543c885b66fcp-3, -0x1.8027c223e1456p-5, 0.0}, \
    {0x1.1f8356f9d1d71p-21, 0x1.3bf3ae516364bp-3, -0x1.694145f1c9e6ep-5, 0.0}, \
    {0x1.0a3e9dc928a62p-22, 0x1.332f3543f529bp-3, -0x1.5478aa2977081p-5, 0.0}, \
    {0x1.e355bbaee85cbp-24, 0x1.2ae9b73ad6f12p-3, -0x1.418846d5a74a1p-5, 0.0}, \
    {0x1.ae07e6041da5ep-25, 0x1.23182513e47c7p-3, -0x1.30361fa0dc4a6p-5, 0.0}, \
    {0x1.77077fc81f8f6p-26, 0x1.1bb0c3fc5dabbp-3, -0x1.20517f00ae159p-5, 0.0}, \
    {0x1.409613d2680bep-27, 0x1.14aaf83496d0ap-3, -0x1.11b120257395ep-5, 0.0}, \
    {0x1.0c9ec5ad0c555p-28, 0x1.0dff1a295b105p-3, -0x1.0431c52a81c97p-5, 0.0}, \
    {0x1.b93de1e27ca3bp-30, 0x1.07a653881e8a4p-3, -0x1.ef6a3d3e292b9p-6, 0.0}, \
    {0x1.6338916169438p-31, 0x1.019a8289a198ap-3, -0x1.d841e020d4957p-6, 0.0}, \
    {0x1.184eb8755fd29p-32, 0x1.f7ac443eb3706p-4, -0x1.c2bcc4f7ed342p-6, 0.0}, \
    {0x1.b1a02a022525ap-34, 0x1.eca86c0660145p-4, -0x1.aeb2f31d95579p-6, 0.0}, \
    {0x1.48c29fcb817c6p-35, 0x1.e22073cc910e7p-4, -0x1.9c014715621b8p-6, 0.0}, \
    {0x1.e8a37a45fc32ep-37, 0x1.d80c2650f5807p-4, -0x1.8a88bb9bee5cbp-6, 0.0}, \
    {0x1.63f16173ac184p-38, 0x1.ce640946d26f3p-4, -0x1.7a2dd30be8d1dp-6, 0.0}, \
    {0x1.fc4bde5e39874p-40, 0x1.c5214859fba35p-4, -0x1.6ad81a61a9a1cp-6, 0.0}, \
    {0x1.63be81e3f6f52p-41, 0x1.bc3da30fb154bp-4, -0x1.5c71c0c224519p-6, 0.0}, \
    {0x1.e817d6c079092p-43, 0x1.b3b35d0d371bcp-4, -0x1.4ee73f96defa2p-6, 0.0}, \
    {0x1.4835bd010a41bp-44, 0x1.ab7d3064369dcp-4, -0x1.4227102ef569dp-6, 0.0}, \
    {0x1.b0a877956b926p-46, 0x1.a39641966c033p-4, -0x1.36216c7bac72fp-6, 0.0}, \
    {0x1.1786a0f6215f0p-47, 0x1.9bfa150fe3ef1p-4, -0x1.2ac818fd5f478p-6, 0.0}, \
    {0x1.62085f435b6a5p-49, 0x1.94a485e216dc8p-4, -0x1.200e365683dc0p-6, 0.0}, \
    {0x1.b7852b203198ap-51, 0x1.8d91bd930e380p-4, -0x1.15e81945cb068p-6, 0.0}, \
    {0x1.0b6c3afdde064p-52, 0x1.86be2cdaf4953p-4, -0x1.0c4b28036e460p-6, 0.0}, \
    {0x1.3efa9e2c21746p-54, 0x1.80268530569f7p-4, -0x1.032dbc2c7be22p-6, 0.0}, \
    {0x1.74f0d4e4e4fbfp-56, 0x1.79c7b30832fecp-4, -0x1.f50e111880e59p-7, 0.0}, \
    {0x1.ab65b268e61ffp-58, 0x1.739ed8b2f9a13p-4, -0x1.e49e0463d5a78p-7, 0.0}, \
    {0x1.e01b4dc58b3b1p-60, 0x1.6da949c2f026dp-4, -0x1.d4fc98b19a82bp-7, 0.0}, \
    {0x1.0851945bd91fcp-61, 0x1.67e486eb3a244p-4, -0x1.c61c4d7ac3500p-7, 0.0}, \
    {0x1.1d461f36f8eccp-63, 0x1.624e3a491a4dcp-4, -0x1.b7f0bc12cb0f5p-7, 0.0}, \
    {0x1.2dcb3a0020f57p-65, 0x1.5ce4340af9ec2p-4, -0x1.aa6e7c1d65df3p-7, 0.0}, \
    {0x1.38f2cee17167dp-67, 0x1.57a4676a6eb5cp-4, -0x1.9d8b0b26fea0bp-7, 0.0}, \
    {0x1.3e16ebd5f938bp-69, 0x1.528ce7efe18f4p-4, -0x1.913cb6f79d8eap-7, 0.0}, \
    {0x1.3ce9b9de78f85p-71, 0x1.4d9be6f7ad9adp-4, -0x1.857a8a471854bp-7, 0.0}, \
    {0x1.357d1c57fda8cp-73, 0x1.48cfb1719720cp-4, -0x1.7a3c3b8634b8cp-7, 0.0}, \
    {0x1.2840eeb0c30acp-75, 0x1.4426add45c753p-4, -0x1.6f7a1d7b2621ep-7, 0.0}, \
    {0x1.15f81e103a069p-77, 0x1.3f9f5a3fe5fc1p-4, -0x1.652d1178df960p-7, 0.0}, \
    {0x1.ff4c323b52532p-80, 0x1.3b384ac942ac1p-4, -0x1.5b4e7b0060f84p-7, 0.0}, \
    {0x1.ccee1660198f4p-82, 0x1.36f027ec300ebp-4, -0x1.51d834a1ab7a9p-7, 0.0}, \
    {0x1.974bd1ce10929p-84, 0x1.32c5ad1e6b0c6p-4, -0x1.48c485f797479p-7, 0.0}, \
    {0x1.60c6cebb31a25p-86, 0x1.2eb7a78174b82p-4, -0x1.400e1a9e83986p-7, 0.0}, \
    {0x1.2b8124c71f30bp-88, 0x1.2ac4f4afd61bcp-4, -0x1.37affa09ebb9ep-7, 0.0}, \
    {0x1.f27bd34319f03p-91, 0x1.26ec81a341c44p-4, -0x1.2fa580206a47ep-7, 0.0}, \
    {0x1.969d47321e4ccp-93, 0x1.232d49b13b244p-4, -0x1.27ea5688b6ba0p-7, 0.0}, \
}
