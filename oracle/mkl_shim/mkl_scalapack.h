/* TEST INFRASTRUCTURE ONLY: empty stand-in for the MKL ScaLAPACK header the
 * reference includes (nothing from it is used). */
