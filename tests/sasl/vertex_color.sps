// The interpolated colour; its only input is linked to whichever varying
// register carries COLOR0.
float4 ps_main(float4 c: COLOR0): SV_Target {
	return c;
}
