/* Empty stand-in: the reference includes this boost header (cpp/soap_snp.h:12-14)
 * but uses nothing from it.  Test infrastructure for oracle/_ref. */
