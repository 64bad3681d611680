/* Stand-in for the reference's generated precision header: the oracle
 * recipe selects the precision with -DdIDESINGLE or -DdIDEDOUBLE. */
#ifndef _ODE_PRECISION_H_
#define _ODE_PRECISION_H_
#if defined(dIDESINGLE)
#define dSINGLE
#elif defined(dIDEDOUBLE)
#define dDOUBLE
#else
#error "define dIDESINGLE or dIDEDOUBLE"
#endif
#endif
